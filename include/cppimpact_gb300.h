/*
 * cppimpact_gb300.h -- C ABI of the GB300-native explicit impact step.
 *
 * One shared library, libcppimpact_gb300.so, exports everything below with C linkage:
 * plain pointers and sizes, no C++ or framework types.  Status codes are int:
 * CI_OK (0) or a negative CI_ERR_*; ci_last_error() returns the message of the last
 * failure on the calling thread.  Host buffers are owned by the caller; device memory
 * is owned by the library and freed by ci_destroy.  One solver is used from one host
 * thread at a time; distinct solvers are independent.
 *
 * The entry points replace the reference's C++ template interface for the hot path
 * (smdogroup/cppimpact, paths relative to the reference checkout):
 *   Dynamics<T,Basis,Analysis,Quadrature>(Mesh*, BaseMaterial*, Wall*)   include/dynamics.h:64-83
 *   Dynamics::initialize(pos, vel)                                       include/dynamics.h:99-111
 *   Dynamics::solve(dt, time_end, export_interval)                       include/dynamics.h:414-512
 *   update<T,3,npe,Basis,Analysis>(...)  (one step's accelerations)      include/dynamics_kernels.h:8-169
 *   FEAnalysis::element_mass_matrix / calculate_f_internal              include/analysis.h:136-162, 321-382
 *   Dynamics::debug_strain (strain energy + volume)                      include/dynamics.h:303-412
 *   Mesh::load_mesh(filename)                                            include/mesh.h:57-267
 * The C++ drop-in headers in include/cppimpact/ keep those class names and
 * signatures and forward to these functions.
 */
#ifndef CPPIMPACT_GB300_H
#define CPPIMPACT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CI_ABI_VERSION 1

/* status codes */
#define CI_OK 0
#define CI_ERR_INVALID -1     /* bad argument or inconsistent mesh */
#define CI_ERR_CUDA -2        /* a CUDA runtime call failed */
#define CI_ERR_DEGENERATE -3  /* an element has det J <= 0 */
#define CI_ERR_NONFINITE -4   /* NaN/Inf appeared in the nodal state */
#define CI_ERR_UNSUPPORTED -5 /* valid request this build does not implement */
#define CI_ERR_IO -6          /* file could not be opened or parsed */
#define CI_ERR_NOMEM -7       /* host or device allocation failed */
#define CI_ERR_TOO_LARGE -8   /* a size limit of the entry point was exceeded */

/* constitutive mode */
#define CI_MODE_J2 0        /* J2 radial return, linear isotropic hardening, stored stress */
#define CI_MODE_REFCOMPAT 1 /* the reference's incremental force K_e(x_n) * (dt v) */

/* mass lumping */
#define CI_LUMP_ROWSUM 0 /* m_i = rho sum_q N_i w_q detJ_q (the reference's rule) */
#define CI_LUMP_HRZ 1    /* Hinton-Rock-Zienkiewicz diagonal scaling (positive for tet10) */

/* Mesh: exactly the fields of Mesh<T,npe> (include/mesh.h:14-18).  Node and element
 * ids are 0-based as after Mesh::load_mesh.  slave/fixed sets are carried for
 * completeness; like the reference wall, contact is tested on every node. */
typedef struct ci_mesh {
  int num_nodes;
  int num_elements;
  int nodes_per_element;    /* 4 (C3D4) or 10 (C3D10, CalculiX edge order) */
  const double* xloc;       /* [3*num_nodes]  x0 y0 z0 x1 ... */
  const int* element_nodes; /* [npe*num_elements] */
  int num_slave_nodes;
  const int* slave_nodes;
  int num_fixed_nodes;
  const int* fixed_nodes;
} ci_mesh;

/* Material: BaseMaterial{E, rho, nu} (include/basematerial.h:6-20) plus the J2
 * parameters Elastoplastic stores (include/elastoplastic.h:7-23).  beta is the
 * kinematic-hardening fraction; only beta = 0 (isotropic) is implemented. */
typedef struct ci_material {
  double E, nu, rho;
  double sigma_y0; /* initial yield stress (Pa); <= 0 or huge means elastic */
  double H;        /* isotropic hardening modulus (Pa): sigma_y = sigma_y0 + H epbar */
  double beta;
} ci_material;

/* Rigid planar wall: contact when d = normal . (x + du) - offset < 0; the node then
 * gets a += -(d k / m) normal.  The reference's Wall<T,dim,Basis>(name, location,
 * stiffness, slave, n, normal) (include/wall.h:23-43) is normal = normal_sign e_dim,
 * offset = normal_sign * location. */
typedef struct ci_wall {
  double normal[3];
  double offset;
  double stiffness; /* N/m */
} ci_wall;

typedef struct ci_options {
  int mode;           /* CI_MODE_* */
  int lumping;        /* CI_LUMP_* */
  double gravity[3];  /* body acceleration; the reference uses (0, 0, -9.81) */
  int device;         /* CUDA device ordinal */
  int chunk_elements; /* elements per CTA chunk, 0 = automatic */
  int chunk_nodes;    /* local-node budget per chunk, 0 = automatic (896; 768 when the
                         task kernel runs) */
  int graph_steps;    /* steps captured per CUDA graph, 0 = automatic */
  int step_kernel;    /* 0 = automatic (2 for four-lane tet10 meshes of more than 0.8 of a
                         round of fused CTAs, else 3), 1 = element + node kernels, 2 = persistent task
                         kernel (tet10, elem_lanes 4, block_threads 128: node and element
                         tasks of all the call's steps), 3 = fused (one launch per step);
                         0, 2 and 3 give the same bits */
  int block_threads;  /* threads per chunk CTA of the fused kernel: 64, 128 or 256; 0 = automatic */
  int elem_lanes;     /* tet10 fused kernel: 4 = one lane per Gauss point, 1 = one thread per
                         element; 0 = automatic (4) */
  int autotune_steps; /* ci_batch_create only: > 0 = time this many steps of candidate tile
                         shapes (chunk_elements, chunk_nodes, block_threads, elem_lanes: those
                         left 0 above) and keep the fastest, see ci_batch_tuning; 0 = none */
} ci_options;

/* energy terms (FP64), see ci_get_energy */
typedef struct ci_energy {
  double kinetic;  /* 1/2 sum m |v_n|^2 at the last completed step */
  double internal; /* sum over steps and QPs of w detJ 1/2 (sigma_n + sigma_{n+1}) : d_eps */
  double plastic;  /* sum over steps and QPs of w detJ sigma_y d_epbar */
  double contact;  /* work done by the wall on the body */
  double gravity;  /* work done by gravity on the body */
  double kinetic0; /* initial kinetic energy */
  double balance;  /* kinetic + internal - contact - gravity - kinetic0 */
} ci_energy;

typedef struct ci_solver ci_solver;

/* ---- library ---- */
int ci_abi_version(void);
const char* ci_last_error(void);
void ci_default_options(ci_options* o);

/* ---- solver lifetime: Dynamics(Mesh*, BaseMaterial*, Wall*), include/dynamics.h:64-83 ---- */
int ci_create(const ci_mesh* mesh, const ci_material* mat, const ci_wall* wall,
              const ci_options* opt, ci_solver** out);
int ci_destroy(ci_solver* s);

/* Dynamics::initialize (include/dynamics.h:99-111): positions X + pos, velocity vel,
 * stored stress and plastic strain zero, contact history cleared. */
int ci_initialize(ci_solver* s, const double pos[3], const double vel[3]);

/* Dynamics::solve (include/dynamics.h:414-512): ci_start (lumped mass, a0 from zero
 * increment, v += dt/2 a0) then steps while time <= time_end (time += dt in double,
 * the reference's loop count).  export_interval is accepted for signature parity;
 * state is read back with ci_get_state. */
int ci_solve(ci_solver* s, double dt, double time_end, int export_interval);

/* Lower-level stepping: ci_start does the mass, a0 and half step of Dynamics::solve
 * from the current positions and velocities (those of ci_initialize or ci_set_state)
 * and clears the stored stress, plastic strain and contact history; ci_step advances
 * nsteps more steps of size dt (graph-captured). */
int ci_start(ci_solver* s, double dt);
int ci_step(ci_solver* s, int nsteps);
int ci_steps_done(const ci_solver* s, long long* nsteps);

/* Read back (any pointer may be NULL): x, v [3N] in the caller's node order (current
 * positions and the half-step velocity held by the reference's vel array), mass [N],
 * sigma [E*nq*6] (Voigt xx yy zz xy yz xz), epbar [E*nq] in the caller's element
 * order (nq = 1 for tet4, 4 for tet10), contact [N]: bit0 in contact at the last
 * step, bit1 ever in contact. */
int ci_get_state(ci_solver* s, double* x, double* v, double* mass, float* sigma, float* epbar,
                 unsigned char* contact);
/* Overwrite the nodal state (caller order, [3N] each); used for restarts. */
int ci_set_state(ci_solver* s, const double* x, const double* v);
/* Deformation gradient F = I + du/dX at every Gauss point of the current state, FP64,
 * [E*nq*9] in the caller's element order, row-major (F[a][j] = delta_aj + du_a/dX_j).
 * The reference computes no F (its update works on the displacement increment,
 * include/dynamics_kernels.h:75-139); this is the reported output of the new
 * deformation-gradient row. */
int ci_deformation_gradient(ci_solver* s, double* F);
/* Nodal output fields of the reference's VTK export (include/dynamics.h:113-254), in the
 * caller's node order; any pointer may be NULL.  acc [3N]: the acceleration of the last
 * completed step (the reference's global_acc).  strain, stress [6N]: the reference's
 * global_strains / global_stress (include/dynamics_kernels.h:117-147): for each element
 * the strain B u of the total displacement u = x - X at the parametric point (0, 0, 0)
 * with B from the current positions, Voigt order xx yy zz gamma_xy gamma_yz gamma_xz,
 * and the elastic stress D strain (include/analysis.h:479-503, tetrahedral.h:442-512);
 * every node takes the value of the last element, in the caller's element order, that
 * contains it.  Computed on the GPU in FP64 on demand (an export-time field, not part
 * of the step). */
int ci_get_nodal_fields(ci_solver* s, double* acc, double* strain, double* stress);
/* Binary state file of a started solver -- the state the reference's export_to_vtk
 * dumps (include/dynamics.h:113-254) plus everything a restart needs: positions,
 * velocities, masses, contact history, stored stress and plastic strain at the Gauss
 * points, energy work sums, dt and the step count.  ci_load_state restores it into a
 * solver created for the same mesh, mode, lumping and chunk options (checked; otherwise
 * CI_ERR_INVALID), after which ci_step continues bit for bit as the saved run would
 * have.  Files are little-endian as written; CI_ERR_IO on open/read/write failures. */
int ci_save_state(ci_solver* s, const char* path);
int ci_load_state(ci_solver* s, const char* path);
int ci_get_energy(ci_solver* s, ci_energy* e);
/* Device status word: bit0 non-positive det J seen, bit1 non-finite state seen. */
int ci_get_status(ci_solver* s, unsigned int* status);

/* ---- one-shot kernels (the per-step seam, include/dynamics_kernels.h:8-169) ---- */
/* Assembled internal force f[3N] of FEAnalysis::calculate_f_internal for positions
 * x[3N] and increment du[3N] on the solver's mesh and mode; sigma_in/epbar_in
 * (caller element order, may be NULL = zero) are the stored QP states, sigma_out /
 * epbar_out (may be NULL) receive the updated ones. */
int ci_internal_force(ci_solver* s, const double* x, const double* du, const float* sigma_in,
                      const float* epbar_in, double* f, float* sigma_out, float* epbar_out);
/* Lumped nodal mass [N] at positions x[3N] (FEAnalysis::element_mass_matrix assembled). */
int ci_lumped_mass(ci_solver* s, const double* x, double* mass);
/* Dynamics::debug_strain: total strain energy 1/2 u . K u and volume at the mesh
 * positions for a prescribed displacement u[3N] (RefCompat force). */
int ci_strain_energy(ci_solver* s, const double* u, double* energy, double* volume);

/* ---- batched solves: many instances of uneven size, one launch per step ----
 * No reference counterpart (the reference solves one mesh per Dynamics object); the
 * batch is the parameter-sweep form of ci_create + ci_initialize + ci_solve.  Every
 * instance has its own mesh (tet4 or tet10), J2 material, wall, initial position
 * offset and velocity, dt and end time; it runs the reference's loop count
 * (while t <= t_end) with HRZ lumping, exactly as a single J2 solve with the same
 * options (bitwise the same result).  Instances of each element type share one
 * graph-captured launch per step; tet4 and tet10 groups run on two streams. */
typedef struct ci_instance {
  ci_mesh mesh;
  ci_material mat;
  ci_wall wall;
  double pos[3];
  double vel[3];
  double dt;
  double t_end;
} ci_instance;
typedef struct ci_batch ci_batch;
int ci_batch_create(const ci_instance* inst, int n, const ci_options* opt, ci_batch** out);
/* Runs every instance from its initial state to its end time; *device_ms (may be
 * NULL) receives the device time of the whole batch (CUDA events). */
int ci_batch_run(ci_batch* b, float* device_ms);
/* Final state of instance i (caller order; any pointer may be NULL): x, v [3N],
 * epbar [E*nq], contact [N] as ci_get_state, *nsteps the steps it ran. */
int ci_batch_get_state(ci_batch* b, int i, double* x, double* v, float* epbar,
                       unsigned char* contact, long long* nsteps);
int ci_batch_destroy(ci_batch* b);
/* Tile shape the batch's group of `npe`-node elements runs with (after autotuning, the
 * winner; trial_ms_per_step its trial time, 0 when not tuned); chunk_elements 0 means
 * each instance's own automatic split.  The shape changes the plan and so the FP32
 * rounding of the results: to reproduce a tuned batch bit for bit, pass the returned
 * shape in ci_options (it then also equals the unbatched run with those options). */
int ci_batch_tuning(ci_batch* b, int npe, int* chunk_elements, int* chunk_nodes, int* block_threads,
                    int* elem_lanes, float* trial_ms_per_step);
/* A run of a batch of one element type that also records the displacement of every
 * node every `every` steps (even) into d_snap [max_snaps][N_total][3] (device FP32,
 * plan order, instances concatenated); snapshot s is the state after (s+1)*every
 * steps.  ci_batch_node_order gives instance i's plan order (perm[p] = caller node)
 * and its offset in N_total. */
int ci_batch_run_snapshots(ci_batch* b, int every, float* d_snap, int max_snaps, float* device_ms);
int ci_batch_node_order(ci_batch* b, int i, int* perm, int* node_offset);
/* Runs the batch like ci_batch_run_snapshots but keeps only, per instance, the largest
 * nodal displacement norm over the same max_snaps snapshot states (FP32, like the
 * snapshots) and the largest equivalent plastic strain of the final state:
 * peak_disp [n], peak_epbar [n] (either may be NULL), in instance order.  The
 * reference has no counterpart (its drivers write VTK files, include/dynamics.h:113-254);
 * this is the sweep's per-run answer without the snapshot buffer. */
int ci_batch_run_peaks(ci_batch* b, int every, int max_snaps, float* peak_disp, float* peak_epbar,
                       float* device_ms);

/* ---- BF16 tensor-core GEMM (surrogate training and inference; no reference
 * counterpart: the reference has no dense contraction) ----
 * C[M x N] = alpha op(A) op(B) + beta C (+ bias[N]) (then tanh if activation == 1) on
 * `stream`.  A, B: BF16 row-major with leading dimensions lda, ldb, transA / transB
 * select op() = transpose.  C: FP32 row-major (ldc); C_bf16 (may be NULL) receives a
 * BF16 copy.  All pointers are device pointers.  *d_error (device int) is set to 1 if
 * a tensor-core wait timed out (the result is then invalid).  When the output has few
 * 128-row tiles and K is long, K is split across CTAs: partial tiles go to a per-device
 * FP32 workspace (one per device and stream, grown by cudaMalloc on first need, at most
 * 32 streams' kept per device) and are summed in a fixed order, so results are
 * deterministic; calls on different streams may run concurrently.  Three paths, all with the same epilogue (alpha, beta C, bias, tanh,
 * BF16 copy): C = A B^T with both operands K-major (transA = 0, transB = 1), M >= 128,
 * N >= 16, K >= 64, 16-byte aligned A and B and leading dimensions that are multiples
 * of 8 runs on a TMA-fed pipelined tensor-core kernel; any other form with at most
 * 2^20 multiply-adds (M N K <= 1048576) runs on the CUDA cores, one thread per output
 * summing the BF16 products in FP32 in K order; the remaining forms run on a
 * tensor-core kernel that stages its operands itself. */
int ci_gemm_bf16(const void* A, int lda, int transA, const void* B, int ldb, int transB, float* C,
                 int ldc, void* C_bf16, int M, int N, int K, float alpha, float beta,
                 const float* bias, int activation, int* d_error, void* stream);

/* ---- surrogate MLP (no reference counterpart) ----
 * n_in -> H -> H -> n_out with tanh hidden layers; every product is ci_gemm_bf16 (BF16
 * operands, FP32 accumulation); FP32 master weights; Adam.  Parameter order:
 * W1 [n_in x H], b1 [H], W2 [H x H], b2 [H], W3 [H x n_out], b3 [n_out] (row-major,
 * a layer computes X W + b).  Data pointers (d_*) are device FP32 row-major. */
typedef struct ci_mlp ci_mlp;
int ci_mlp_create(int n_in, int n_hidden, int n_out, unsigned long long seed, ci_mlp** out);
int ci_mlp_destroy(ci_mlp* m);
long long ci_mlp_num_params(const ci_mlp* m);
int ci_mlp_set_params(ci_mlp* m, const float* h_params);
int ci_mlp_get_params(ci_mlp* m, float* h_params);
/* d_Y [n x n_out] = MLP(d_X [n x n_in]) */
int ci_mlp_predict(ci_mlp* m, const float* d_X, int n, float* d_Y, void* stream);
/* gradients of the mean squared error over all n rows into h_grad [num_params] (host) */
int ci_mlp_gradients(ci_mlp* m, const float* d_X, const float* d_T, int n, float* h_grad,
                     double* loss);
/* epochs of mini-batch Adam (seeded shuffles); h_loss [epochs] (may be NULL) receives the
 * last mini-batch loss of each epoch */
int ci_mlp_train(ci_mlp* m, const float* d_X, const float* d_T, int n, int batch, int epochs,
                 float lr, unsigned long long seed, double* h_loss, void* stream);

/* ---- allocation-free variant (no counterpart in the reference) ----
 * ci_strain_energy_noalloc computes what ci_strain_energy computes -- the total strain
 * energy 1/2 u.K u and the volume of a mesh for a prescribed displacement -- without
 * allocating anything, for callers that cannot call cudaMalloc: programs that own all
 * device memory through their own pool and forbid driver allocations after start-up,
 * plug-ins living inside such programs, and time-critical loops that must not incur
 * cudaMalloc's synchronisation or its failure under memory pressure.  It needs no
 * solver: d_xloc [3N] and d_u [3N] (FP64), d_element_nodes [npe*E] (int) and d_out [2]
 * (energy, volume; FP64) are device buffers the caller owns; the work is enqueued on
 * `stream` (a cudaStream_t, NULL = the legacy default stream) and the result is in
 * d_out once that stream reaches it.  Its scratch is a fixed array compiled into the
 * library (CI_NOALLOC_MAX_ELEMENTS / 256 blocks x 2 doubles = 256 KiB on every GPU the
 * library is used on), so at most CI_NOALLOC_MAX_ELEMENTS elements are accepted
 * (CI_ERR_TOO_LARGE beyond).  The first call on each device looks up the scratch's
 * device address and should happen before any stream capture; that address is kept
 * for the life of the device's primary context, so after cudaDeviceReset the entry
 * point must not be called again in the same process.  Calls share the scratch:
 * calls that can overlap on the GPU race and must be serialised by the caller.  A
 * non-positive det J makes the energy NaN; a node index outside [0, num_nodes) makes
 * the energy and the volume NaN (that element's loads are skipped). */
#define CI_NOALLOC_MAX_ELEMENTS (1 << 22)
int ci_strain_energy_noalloc(const double* d_xloc, const int* d_element_nodes, int num_nodes,
                             int num_elements, int nodes_per_element, const double* d_u, double E,
                             double nu, double* d_out, void* stream);

/* ---- timing helpers for benchmarks (CUDA events on the solver's stream) ---- */
int ci_time_steps(ci_solver* s, int nsteps, float* ms);
/* Runs nsteps steps launching each kernel between CUDA events and returns mean device
 * durations (ms): fused path out[0] = the step kernel, out[1] = the one end-of-call
 * finalise divided by nsteps (its share per step); two-kernel path out[0] = element
 * kernel, out[1] = node kernel. */
int ci_time_kernels(ci_solver* s, int nsteps, float* out_ms);
/* Kernel launches one step issues (for launch accounting; the task kernel launches once
 * per call of up to 65,536 steps). */
int ci_launches_per_step(const ci_solver* s);
/* The step kernel a solver runs (ci_options::step_kernel with 0 resolved), -1 for NULL. */
int ci_step_kernel(const ci_solver* s);

/* Test hook for the task kernel's bounded waits: in the next launch (the next ci_step /
 * ci_solve call) chunk `chunk` never publishes its progress, so the tasks waiting for it
 * give up after wait_seconds (0 < wait_seconds <= 60), set the abort flag for the others
 * and the call returns CI_ERR_CUDA ("a task waited longer than its time limit") with the
 * CUDA context intact; the solver's state is then partial.  CI_ERR_UNSUPPORTED unless
 * the solver runs the task kernel. */
int ci_debug_flow_stall(ci_solver* s, int chunk, double wait_seconds);

/* ---- mesh utilities (host only) ---- */
/* Mesh::load_mesh (include/mesh.h:57-267): parse an Abaqus/CalculiX .inp file.
 * Arrays are malloc'ed by the library and released with ci_mesh_free. */
int ci_mesh_load_inp(const char* path, int nodes_per_element, ci_mesh* out);
void ci_mesh_free(ci_mesh* m);

/* Preprocessing summary (host only, no GPU needed): space-filling-curve order,
 * chunking, node ownership and per-chunk colouring.  stats[0..7] = chunks,
 * max colours, max local nodes, total slots, max chunk elements, ghosts, boundary
 * nodes, the longest dependency list of the task kernel (chunks a chunk's element task
 * or node task waits for). perm_elems (may be NULL, [E]) receives the plan order of elements
 * (original ids), perm_nodes (may be NULL, [N]) the plan order of nodes. */
int ci_plan_stats(const ci_mesh* mesh, int chunk_elements, int chunk_nodes, long long* stats,
                  int* perm_elems, int* perm_nodes);
/* Check a plan's invariants on the host: every element once, colours conflict-free
 * within each chunk, slot lists cover every (chunk, node) pair, and the task kernel's
 * dependency lists (each chunk's node owners and their transpose) and chunk task order
 * are complete and consistent.  Returns CI_OK. */
int ci_plan_verify(const ci_mesh* mesh, int chunk_elements, int chunk_nodes);

#ifdef __cplusplus
}
#endif
#endif /* CPPIMPACT_GB300_H */
