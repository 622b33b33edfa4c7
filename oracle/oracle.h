/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 CPU oracle for the explicit tet4/tet10 impact step.  Only tests/, the smoke
 * check in __graft_entry__.py and bench.py's CPU-baseline / reference legs may load
 * liboracle.so, and only as the checker or the timed CPU baseline.  The product
 * library (libcppimpact_gb300.so) never links or calls anything here.
 *
 * Two independent restatements live behind this header:
 *
 *  1. orc_ref_*  (ref_port.cpp) -- a restatement of smdogroup/cppimpact's CPU path:
 *     Dynamics::solve (include/dynamics.h:414-512), update (include/dynamics_kernels.h:8-169),
 *     FEAnalysis::element_mass_matrix / calculate_f_internal / calculate_stress_strain /
 *     calculate_strain_energy / calculate_volume (include/analysis.h:136-162, 321-503),
 *     the tet4/tet10 bases and the truncated 5-point rule (include/tetrahedral.h:7-41,
 *     182-269, 442-512, 515-657), inv3x3 (include/physics.h:38-58) and
 *     Wall::detect_contact (include/wall.h:37-43).  Same formulas, same quadrature
 *     constants, same accumulation order, so it reproduces the reference to round-off.
 *     Its parity is pinned against the compiled reference (oracle/_ref) through
 *     tests/golden/ fixtures.
 *
 *  2. orc_*      (solver64.cpp) -- the FP64 restatement of the GB300 solver's own
 *     formulation: matrix-free internal force with 1 (tet4) / 4 (tet10) Gauss points,
 *     J2 radial return with linear isotropic hardening (Simo & Hughes 1998, Box 3.1),
 *     row-sum or HRZ lumping, planar penalty wall, FP64 energy terms.  With
 *     mode = ORC_REFCOMPAT it computes the reference's force K_e(x_n) * (dt v) and is
 *     checked against (1); the J2 mode is pinned by closed-form material-point tests
 *     and the elastic-limit identity J2(sigma_y -> inf, sigma_n = 0) == RefCompat.
 */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mesh {
  int num_nodes;
  int num_elements;
  int nodes_per_element; /* 4 or 10 */
  const double* xloc;    /* [3*num_nodes], x0 y0 z0 x1 ... */
  const int* conn;       /* [npe*num_elements], 0-based */
} orc_mesh;

/* ------------------------------------------------------------------ */
/* 1. Reference restatement                                             */
/* ------------------------------------------------------------------ */
typedef struct orc_ref_params {
  double E, nu, rho;
  int wall_dim;           /* axis the wall is normal to (the reference uses 2) */
  double wall_location;   /* Wall::location */
  double wall_stiffness;  /* Wall::stiffness */
  int wall_normal;        /* +1 / -1 */
  int gravity_dim;        /* 2 in the reference */
  double gravity;         /* -9.81 in the reference */
} orc_ref_params;

/* Row-sum lumped mass with the truncated 5-point rule, assembled in element order
 * (include/analysis.h:136-162, include/dynamics_kernels.h:36-73).  mass[3*N]. */
int orc_ref_lumped_mass(const orc_mesh* m, double rho, const double* xloc, double* mass3);

/* One call of the reference's per-step update (include/dynamics_kernels.h:8-169):
 * acc[3N] from the current positions xloc, the increment dof and the assembled
 * mass3[3N] (assembled here first when mass3[0] == 0, as the reference does).
 * xloc0 are the undeformed positions used for the stress/strain output; strains and
 * stress ([6N], last writer wins) may be NULL.  nthreads > 1 splits the element
 * loop into contiguous ranges whose per-thread accelerations are summed in thread
 * order (deterministic; identical to nthreads = 1 up to summation order). */
int orc_ref_update(const orc_mesh* m, const orc_ref_params* p, const double* xloc0,
                   const double* xloc, const double* dof, double* acc, double* mass3,
                   double* strains, double* stress, int nthreads);

/* The whole staggered central-difference solve of Dynamics::solve
 * (include/dynamics.h:414-512) after Dynamics::initialize (include/dynamics.h:99-111).
 * The loop runs while time <= time_end with time += dt in double, exactly like the
 * reference.  Outputs (any may be NULL): x_out[3N] current positions, v_out[3N]
 * velocities, mass_out[3N], acc_out[3N]; *nsteps_out the number of loop iterations. */
int orc_ref_solve(const orc_mesh* m, const orc_ref_params* p, const double init_pos[3],
                  const double init_vel[3], double dt, double time_end, int nthreads,
                  double* x_out, double* v_out, double* mass_out, double* acc_out,
                  int* nsteps_out);

/* Dynamics::debug_strain (include/dynamics.h:303-412): prescribed displacement
 * case 0: (a x, -nu a x, -nu a x); case 1: (a x^2/2, -nu a x^2/2, -nu a x^2/2).
 * Returns the total strain energy and volume the reference prints. */
int orc_ref_debug_strain(const orc_mesh* m, double E, double nu, double alpha, int def_case,
                         double* energy, double* volume);

/* ------------------------------------------------------------------ */
/* 2. FP64 oracle of the GB300 solver's formulation                    */
/* ------------------------------------------------------------------ */
enum { ORC_J2 = 0, ORC_REFCOMPAT = 1 };
enum { ORC_LUMP_ROWSUM = 0, ORC_LUMP_HRZ = 1 };

typedef struct orc_params {
  double E, nu, rho;
  double sigma_y0, H;     /* J2 yield stress and isotropic hardening modulus */
  int mode;               /* ORC_J2 / ORC_REFCOMPAT */
  int lumping;            /* ORC_LUMP_ROWSUM / ORC_LUMP_HRZ */
  double wall_normal[3];  /* unit normal of the wall plane, pointing into the body */
  double wall_offset;     /* plane: normal . x = offset */
  double wall_stiffness;  /* penalty stiffness (N/m) */
  double gravity[3];
} orc_params;

/* energy[] layout of orc_get */
enum {
  ORC_E_KINETIC = 0,   /* 1/2 sum m |v_n|^2 with v_n = v_{n+1/2} - dt/2 a_n */
  ORC_E_INTERNAL = 1,  /* sum_q w detJ 1/2 (sigma_n + sigma_{n+1}) : d_eps */
  ORC_E_PLASTIC = 2,   /* sum_q w detJ sigma_y(epbar) d_epbar */
  ORC_E_CONTACT = 3,   /* work done by the wall on the body */
  ORC_E_GRAVITY = 4,   /* work done by gravity on the body */
  ORC_E_KINETIC0 = 5,  /* initial kinetic energy */
  ORC_E_BALANCE = 6,   /* KE + W_int - W_contact - W_gravity - KE0 */
  ORC_E_COUNT = 8
};

int orc_num_qp(int npe); /* 1 for tet4, 4 for tet10 */

/* Lumped nodal mass of the GB300 formulation: mass[N]. */
int orc_lumped_mass(const orc_mesh* m, const orc_params* p, const double* xloc, double* mass);

/* One-shot assembled internal force f[3N] for positions x[3N] and increment du[3N].
 * sigma_in/epbar_in ([E][nq][6], [E][nq]) are the stored QP states (NULL = zero);
 * sigma_out/epbar_out (may be NULL) receive the updated states.  mode/material
 * from p.  Returns the internal-work and plastic-dissipation increments in
 * work[2] when work != NULL. */
int orc_internal_force(const orc_mesh* m, const orc_params* p, const double* x,
                       const double* du, const double* sigma_in, const double* epbar_in,
                       double* f, double* sigma_out, double* epbar_out, double* work);

/* J2 radial return at one material point (Voigt xx yy zz xy yz xz; engineering
 * shear strains in d_eps).  sigma[6] and *epbar updated in place. */
void orc_j2_update(double E, double nu, double sigma_y0, double H, const double d_eps[6],
                   double sigma[6], double* epbar);

typedef struct orc_solver orc_solver;
orc_solver* orc_create(const orc_mesh* m, const orc_params* p);
void orc_destroy(orc_solver* s);
/* x = X + pos, v = vel; mass; a0 from zero increment; v += dt/2 a0 (dynamics.h:440-463) */
int orc_initialize(orc_solver* s, const double pos[3], const double vel[3], double dt);
int orc_step(orc_solver* s, int nsteps);
/* Threads of orc_step's loops (default 1).  The results do not depend on it: each
 * node's force is summed over its elements in element order, as with one thread, and
 * the work terms over fixed blocks of elements in block order. */
int orc_set_threads(orc_solver* s, int nthreads);
/* Any output may be NULL.  x, v: [3N]; mass [N]; sigma [E*nq*6]; epbar [E*nq];
 * energy [ORC_E_COUNT]; contact [N]: bit0 in contact at the last step, bit1 ever. */
int orc_get(const orc_solver* s, double* x, double* v, double* mass, double* sigma,
            double* epbar, double* energy, unsigned char* contact);

#ifdef __cplusplus
}
#endif
