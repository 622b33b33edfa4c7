// ci_solver.cu -- C ABI of the GB300 impact step (declared in include/cppimpact_gb300.h).
//
// Host orchestration: preprocessing (ci_plan.cpp), device buffers, the one-time
// lumped mass and initial half step, graph-captured stepping, read-back in the
// caller's node/element order, one-shot kernels for parity checks.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/cppimpact_gb300.h"
#include "ci_kernels.cuh"
#include "ci_plan.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define CI_CUDA(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(CI_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                  __FILE__, __LINE__);                                                     \
  } while (0)

constexpr int kBS = 256;
// local-node budget per chunk of the task kernel when the budget is automatic
constexpr int kTaskChunkNodes = 768;

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, sizeof(T) * count);
  }
};

}  // namespace

namespace ci {
// Sets the message returned by ci_last_error on this thread (used by other files of
// the library) and passes the status code through.
int set_last_error(int code, const char* msg) {
  g_last_error = msg;
  return code;
}
}  // namespace ci

struct ci_solver {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ci::Plan plan;
  int N = 0, E = 0, npe = 0, nq = 0, C = 0;
  long long S = 0, Lt = 0;
  ci_material mat{};
  ci_wall wall{};
  ci_options opt{};
  std::vector<double> X0;   // mesh positions, caller order [3N]
  std::vector<double> X;    // reference positions X0 + pos, caller order
  std::vector<double> vel0; // initial velocity
  double dt = 0.0;
  bool started = false;
  long long steps_done = 0;
  size_t smem_bytes = 0;

  // device plan
  DBuf<ci::ChunkInfo> d_chunks;
  DBuf<uint16_t> d_conn;
  DBuf<uint8_t> d_color;
  DBuf<int> d_lgid, d_lslot, d_slot_row, d_lsrow;
  DBuf<float> d_lx0;  // [3][Lt]
  // state (A buffer = d_u/d_v always holds the state between calls; B is the fused
  // path's second buffer)
  DBuf<double> d_u, d_v;   // [3][N]
  DBuf<double> d_ub, d_vb; // [3][N]
  DBuf<float> d_halo1;     // [3][S] second halo buffer of the fused path
  DBuf<float> d_slot;      // [3][S]
  DBuf<float> d_mass;      // [N]
  DBuf<double> d_d0;       // [N]
  DBuf<float> d_d0f;       // [N]
  DBuf<unsigned char> d_contact;
  DBuf<float> d_acc;       // [3][N]
  DBuf<float4> d_sig_a;
  DBuf<float2> d_sig_b;
  DBuf<float> d_epbar;
  DBuf<double> d_work;     // [C][4]
  DBuf<unsigned int> d_status;
  // one-shot scratch (never aliases the running state)
  DBuf<double> d_u2, d_v2, d_f;
  DBuf<float4> d_sig_a2;
  DBuf<float2> d_sig_b2;
  DBuf<float> d_epbar2;
  DBuf<double> d_epart;
  // caller-order exchange of x and v (allocated on first use): reference positions and
  // the plan index of every caller node, and [3N] AoS staging buffers
  DBuf<double> d_Xc, d_xc, d_vc;
  DBuf<int> d_node_new;
  // persistent task kernel (step_kernel = 2): node records of the two parities, the
  // owner / toucher lists of every chunk, per-chunk progress counters, the task counter
  // and the abort flag ([2C + 2] ints), and the CTAs it keeps resident
  DBuf<float4> d_rec;  // task kernel records: [2][N] float4 then [2][N] float2
  DBuf<int> d_flow_desc, d_flow_ctr;
  int flow_ctas = 0, flow_stride = 0;
  unsigned long long flow_wait_ns = ci::kFlowWaitNs;
  int flow_stall_chunk = -1;  // test hook, for the next task-kernel launch only
  size_t flow_smem = 0;
  bool xc_stale = true;  // X changed since d_Xc was uploaded
  // nodal strain/stress output: last element (caller order) of every node, and the plan
  // position of every caller element (built on first use)
  std::vector<int> last_elem, elem_new;

  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  cudaGraphExec_t graph_cont = nullptr;  // fused path: a block that continues a chained one

  ci::DevPlan dev_plan() const {
    ci::DevPlan P;
    P.chunks = d_chunks.p;
    P.conn_local = d_conn.p;
    P.color = d_color.p;
    P.local_gid = d_lgid.p;
    P.local_slot = d_lslot.p;
    P.local_srow = reinterpret_cast<const int2*>(d_lsrow.p);
    P.local_x0 = d_lx0.p;
    P.slot_row = d_slot_row.p;
    P.E = E;
    P.N = N;
    P.Lt = (int)Lt;
    return P;
  }
  ci::DevState dev_state(double* u, double* v) const {
    ci::DevState D;
    for (int k = 0; k < 3; k++) {
      D.u[k] = u + (size_t)k * N;
      D.v[k] = v + (size_t)k * N;
      D.slot_f[k] = d_slot.p + (size_t)k * S;
    }
    D.sig_a = d_sig_a.p;
    D.sig_b = d_sig_b.p;
    D.epbar = d_epbar.p;
    D.chunk_work = d_work.p;
    D.status = d_status.p;
    D.inst_ep = nullptr;
    return D;
  }
  ci::ElemParams elem_params(float dtf, bool energy) const {
    ci::ElemParams p;
    p.dt = dtf;
    p.mu = (float)(mat.E / (2.0 * (1.0 + mat.nu)));
    p.lambda = (float)(mat.E * mat.nu / ((1.0 + mat.nu) * (1.0 - 2.0 * mat.nu)));
    const bool elastic = !(mat.sigma_y0 > 0.0) || mat.sigma_y0 > 1e30;
    p.sy0 = elastic ? 3.0e38f : (float)mat.sigma_y0;
    p.H = (float)mat.H;
    p.rho = (float)mat.rho;
    p.accum_energy = energy ? 1 : 0;
    return p;
  }
  ci::NodeArrays node_arrays() const {
    ci::NodeArrays A;
    for (int k = 0; k < 3; k++) {
      A.u[k] = d_u.p + (size_t)k * N;
      A.v[k] = d_v.p + (size_t)k * N;
      A.slot_f[k] = d_slot.p + (size_t)k * S;
      A.acc[k] = d_acc.p + (size_t)k * N;
    }
    A.slot_row = d_slot_row.p;
    A.mass = d_mass.p;
    A.d0 = d_d0.p;
    A.contact = d_contact.p;
    A.status = d_status.p;
    return A;
  }
  ci::FusedArgs fused_args(bool cur_is_a, int halo_cur, bool state_final, bool store_acc) const {
    ci::FusedArgs F;
    F.P = dev_plan();
    double* ua = d_u.p;
    double* va = d_v.p;
    double* ub = d_ub.p;
    double* vb = d_vb.p;
    float* h[2] = {d_slot.p, d_halo1.p};
    for (int k = 0; k < 3; k++) {
      F.u_cur[k] = (cur_is_a ? ua : ub) + (size_t)k * N;
      F.v_cur[k] = (cur_is_a ? va : vb) + (size_t)k * N;
      F.u_prv[k] = (cur_is_a ? ub : ua) + (size_t)k * N;
      F.v_prv[k] = (cur_is_a ? vb : va) + (size_t)k * N;
      F.halo_cur[k] = h[halo_cur] + (size_t)k * S;
      F.halo_prv[k] = h[halo_cur ^ 1] + (size_t)k * S;
      F.acc[k] = d_acc.p + (size_t)k * N;
    }
    F.mass = d_mass.p;
    F.d0 = d_d0.p;
    F.d0f = d_d0f.p;
    F.contact = d_contact.p;
    F.sig_a = d_sig_a.p;
    F.sig_b = d_sig_b.p;
    F.epbar = d_epbar.p;
    F.chunk_work = d_work.p;
    F.status = d_status.p;
    F.state_final = state_final ? 1 : 0;
    F.store_acc = store_acc ? 1 : 0;
    F.inst_ep = nullptr;
    F.inst_np = nullptr;
    F.inst_nsteps = nullptr;
    F.step_ctr = nullptr;
    F.step_off = 0;
    return F;
  }
  ci::NodeParams node_params() const {
    ci::NodeParams p;
    p.dt = dt;
    for (int k = 0; k < 3; k++) {
      p.g[k] = opt.gravity[k];
      p.wall_n[k] = wall.normal[k];
      p.gf[k] = (float)opt.gravity[k];
      p.nf[k] = (float)wall.normal[k];
    }
    p.wall_k = wall.stiffness;
    p.N = N;
    return p;
  }
};

namespace {

template <int NPE, int MODE>
cudaError_t launch_elem(ci_solver* s, const ci::DevState& D, const ci::ElemParams& p) {
  ci::k_elem<NPE, MODE, kBS><<<s->C, kBS, s->smem_bytes, s->stream>>>(s->dev_plan(), D, p);
  return cudaGetLastError();
}

template <int NPE, int BS>
cudaError_t configure_step(int bytes) {
  cudaError_t e = cudaFuncSetAttribute(ci::k_step<NPE, ci::EM_J2, BS>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e) return e;
  if (NPE == 10) {
    if ((e = cudaFuncSetAttribute(ci::k_step_t10<ci::EM_J2, BS>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
      return e;
    if ((e = cudaFuncSetAttribute(ci::k_step_t10<ci::EM_REFCOMPAT, BS>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
      return e;
    if ((e = cudaFuncSetAttribute(ci::k_step_qp10<ci::EM_J2, BS>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
      return e;
    if ((e = cudaFuncSetAttribute(ci::k_step_qp10<ci::EM_REFCOMPAT, BS>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
      return e;
  }
  return cudaFuncSetAttribute(ci::k_step<NPE, ci::EM_REFCOMPAT, BS>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// Raise the dynamic shared-memory limit of the element kernels once per solver (not
// inside stream capture).
template <int NPE>
cudaError_t configure_npe(int bytes) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(ci::k_elem<NPE, ci::EM_J2, kBS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
    return e;
  if ((e = cudaFuncSetAttribute(ci::k_elem<NPE, ci::EM_REFCOMPAT, kBS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
    return e;
  if ((e = cudaFuncSetAttribute(ci::k_elem<NPE, ci::EM_MASS_ROWSUM, kBS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
    return e;
  if ((e = configure_step<NPE, 64>(bytes))) return e;
  if ((e = configure_step<NPE, 128>(bytes))) return e;
  if ((e = configure_step<NPE, 256>(bytes))) return e;
  return cudaFuncSetAttribute(ci::k_elem<NPE, ci::EM_MASS_HRZ, kBS>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int NPE, int BS>
cudaError_t launch_fused_bs(ci_solver* s, const ci::FusedArgs& F, const ci::ElemParams& ep,
                            const ci::NodeParams& np) {
  if (NPE == 10 && s->opt.elem_lanes == 4) {
    if (s->opt.mode != CI_MODE_REFCOMPAT)
      ci::k_step_qp10<ci::EM_J2, BS><<<s->C, BS, s->smem_bytes, s->stream>>>(F, ep, np);
    else
      ci::k_step_qp10<ci::EM_REFCOMPAT, BS><<<s->C, BS, s->smem_bytes, s->stream>>>(F, ep, np);
    return cudaGetLastError();
  }
  if (NPE == 10) {
    if (s->opt.mode != CI_MODE_REFCOMPAT)
      ci::k_step_t10<ci::EM_J2, BS><<<s->C, BS, s->smem_bytes, s->stream>>>(F, ep, np);
    else
      ci::k_step_t10<ci::EM_REFCOMPAT, BS><<<s->C, BS, s->smem_bytes, s->stream>>>(F, ep, np);
    return cudaGetLastError();
  }
  if (s->opt.mode != CI_MODE_REFCOMPAT)
    ci::k_step<NPE, ci::EM_J2, BS><<<s->C, BS, s->smem_bytes, s->stream>>>(F, ep, np);
  else
    ci::k_step<NPE, ci::EM_REFCOMPAT, BS><<<s->C, BS, s->smem_bytes, s->stream>>>(F, ep, np);
  return cudaGetLastError();
}

cudaError_t launch_fused(ci_solver* s, const ci::FusedArgs& F) {
  const ci::ElemParams ep = s->elem_params((float)s->dt, true);
  const ci::NodeParams np = s->node_params();
  const int bs = s->opt.block_threads;
  if (s->npe == 4) {
    if (bs == 64) return launch_fused_bs<4, 64>(s, F, ep, np);
    if (bs == 128) return launch_fused_bs<4, 128>(s, F, ep, np);
    return launch_fused_bs<4, 256>(s, F, ep, np);
  }
  if (bs == 64) return launch_fused_bs<10, 64>(s, F, ep, np);
  if (bs == 128) return launch_fused_bs<10, 128>(s, F, ep, np);
  return launch_fused_bs<10, 256>(s, F, ep, np);
}

cudaError_t launch_finalize(ci_solver* s, const ci::FusedArgs& F) {
  ci::k_finalize_nodes<<<(s->N + 255) / 256, 256, 0, s->stream>>>(F, s->node_params());
  return cudaGetLastError();
}

// n fused steps.  start_final: the complete state S^0 is in buffer A (else S^{-1} is in
// buffer B with the halo of the step before; the blocks of even length that chain
// without completing the nodes leave it so).  finish: complete S^n into buffer A.
cudaError_t enqueue_fused(ci_solver* s, int n, bool start_final = true, bool finish = true) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e;
  for (int i = 0; i < n; i++) {
    const ci::FusedArgs F = s->fused_args((i & 1) == 0, i & 1, i == 0 && start_final, false);
    if ((e = launch_fused(s, F))) return e;
  }
  if (!finish) return cudaSuccess;
  // S^n from S^{n-1} (prv) and the halo of step n-1 (with the accelerations a^n)
  const ci::FusedArgs F = s->fused_args((n & 1) == 0, n & 1, false, true);
  if ((e = launch_finalize(s, F))) return e;
  if (n & 1) {
    const size_t b = sizeof(double) * 3 * (size_t)s->N;
    if ((e = cudaMemcpyAsync(s->d_u.p, s->d_ub.p, b, cudaMemcpyDeviceToDevice, s->stream))) return e;
    if ((e = cudaMemcpyAsync(s->d_v.p, s->d_vb.p, b, cudaMemcpyDeviceToDevice, s->stream))) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_elem_mode(ci_solver* s, int mode, const ci::DevState& D, const ci::ElemParams& p) {
  if (s->npe == 4) {
    switch (mode) {
      case ci::EM_J2: return launch_elem<4, ci::EM_J2>(s, D, p);
      case ci::EM_REFCOMPAT: return launch_elem<4, ci::EM_REFCOMPAT>(s, D, p);
      case ci::EM_MASS_ROWSUM: return launch_elem<4, ci::EM_MASS_ROWSUM>(s, D, p);
      default: return launch_elem<4, ci::EM_MASS_HRZ>(s, D, p);
    }
  }
  switch (mode) {
    case ci::EM_J2: return launch_elem<10, ci::EM_J2>(s, D, p);
    case ci::EM_REFCOMPAT: return launch_elem<10, ci::EM_REFCOMPAT>(s, D, p);
    case ci::EM_MASS_ROWSUM: return launch_elem<10, ci::EM_MASS_ROWSUM>(s, D, p);
    default: return launch_elem<10, ci::EM_MASS_HRZ>(s, D, p);
  }
}

int step_mode(const ci_solver* s) {
  return s->opt.mode == CI_MODE_REFCOMPAT ? ci::EM_REFCOMPAT : ci::EM_J2;
}

// One time step: K1 then K2.
cudaError_t enqueue_step(ci_solver* s, bool store_acc) {
  const ci::DevState D = s->dev_state(s->d_u.p, s->d_v.p);
  cudaError_t e = launch_elem_mode(s, step_mode(s), D, s->elem_params((float)s->dt, true));
  if (e != cudaSuccess) return e;
  const int nb = (s->N + 255) / 256;
  if (store_acc)
    ci::k_node<false, true><<<nb, 256, 0, s->stream>>>(s->node_arrays(), s->node_params());
  else
    ci::k_node<false, false><<<nb, 256, 0, s->stream>>>(s->node_arrays(), s->node_params());
  return cudaGetLastError();
}

int check_status(ci_solver* s) {
  unsigned int st = 0;
  CI_CUDA(cudaMemcpyAsync(&st, s->d_status.p, sizeof(st), cudaMemcpyDeviceToHost, s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  if (st & ci::ST_DEGENERATE) return fail(CI_ERR_DEGENERATE, "an element has det J <= 0");
  if (st & ci::ST_NONFINITE) return fail(CI_ERR_NONFINITE, "non-finite nodal state");
  if (st & ci::ST_FLOW_TIMEOUT)
    return fail(CI_ERR_CUDA, "step task kernel: a task waited longer than its time limit");
  return CI_OK;
}

// Per-chunk reference coordinates relative to the chunk origin (first owned node, or
// the first local node), and the wall offsets d0 = n . X - offset, in plan order.
int upload_reference(ci_solver* s) {
  const ci::Plan& P = s->plan;
  std::vector<float> lx0(3 * (size_t)s->Lt);
  for (int c = 0; c < s->C; c++) {
    const ci::ChunkInfo& ch = P.chunks[c];
    const int o = P.node_orig[P.local_gid[ch.local_begin]];
    for (int l = 0; l < ch.n_local; l++) {
      const int lb = ch.local_begin + l;
      const int n = P.node_orig[P.local_gid[lb]];
      for (int k = 0; k < 3; k++)
        lx0[(size_t)k * s->Lt + lb] = (float)(s->X[3 * (size_t)n + k] - s->X[3 * (size_t)o + k]);
    }
  }
  std::vector<double> d0(s->N);
  for (int i = 0; i < s->N; i++) {
    const int n = P.node_orig[i];
    d0[i] = s->wall.normal[0] * s->X[3 * (size_t)n] + s->wall.normal[1] * s->X[3 * (size_t)n + 1] +
            s->wall.normal[2] * s->X[3 * (size_t)n + 2] - s->wall.offset;
  }
  CI_CUDA(cudaMemcpyAsync(s->d_lx0.p, lx0.data(), sizeof(float) * lx0.size(),
                          cudaMemcpyHostToDevice, s->stream));
  CI_CUDA(cudaMemcpyAsync(s->d_d0.p, d0.data(), sizeof(double) * d0.size(), cudaMemcpyHostToDevice,
                          s->stream));
  std::vector<float> d0f(d0.begin(), d0.end());
  CI_CUDA(cudaMemcpyAsync(s->d_d0f.p, d0f.data(), sizeof(float) * d0f.size(), cudaMemcpyHostToDevice,
                          s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  return CI_OK;
}

// u = 0 and v = the initial velocity everywhere.
int reset_kinematics(ci_solver* s) {
  const int N = s->N;
  std::vector<double> v(3 * (size_t)N);
  for (int i = 0; i < N; i++)
    for (int k = 0; k < 3; k++) v[(size_t)k * N + i] = s->vel0[k];
  CI_CUDA(cudaMemsetAsync(s->d_u.p, 0, sizeof(double) * 3 * N, s->stream));
  CI_CUDA(cudaMemcpyAsync(s->d_v.p, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice,
                          s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  return CI_OK;
}

// Stored stress, plastic strain, contact history, work sums and status cleared.
int reset_history(ci_solver* s) {
  const int N = s->N;
  if (s->d_sig_a.p) {
    CI_CUDA(cudaMemsetAsync(s->d_sig_a.p, 0, sizeof(float4) * s->d_sig_a.n, s->stream));
    CI_CUDA(cudaMemsetAsync(s->d_sig_b.p, 0, sizeof(float2) * s->d_sig_b.n, s->stream));
    CI_CUDA(cudaMemsetAsync(s->d_epbar.p, 0, sizeof(float) * s->d_epbar.n, s->stream));
  }
  CI_CUDA(cudaMemsetAsync(s->d_contact.p, 0, N, s->stream));
  CI_CUDA(cudaMemsetAsync(s->d_acc.p, 0, sizeof(float) * 3 * N, s->stream));
  CI_CUDA(cudaMemsetAsync(s->d_work.p, 0, sizeof(double) * 4 * s->C, s->stream));
  CI_CUDA(cudaMemsetAsync(s->d_status.p, 0, sizeof(unsigned int), s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  s->started = false;
  s->steps_done = 0;
  return CI_OK;
}

int reset_state(ci_solver* s) {
  const int rc = reset_kinematics(s);
  return rc ? rc : reset_history(s);
}

int compute_mass(ci_solver* s) {
  const ci::DevState D = s->dev_state(s->d_u.p, s->d_v.p);
  const int mode = s->opt.lumping == CI_LUMP_HRZ ? ci::EM_MASS_HRZ : ci::EM_MASS_ROWSUM;
  CI_CUDA(launch_elem_mode(s, mode, D, s->elem_params(0.f, false)));
  ci::k_mass_sum<<<(s->N + 255) / 256, 256, 0, s->stream>>>(s->d_slot.p, s->d_slot_row.p,
                                                            s->d_mass.p, s->N);
  CI_CUDA(cudaGetLastError());
  return CI_OK;
}

void destroy_graph(ci_solver* s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->graph_cont) cudaGraphExecDestroy(s->graph_cont);
  s->graph = nullptr;
  s->graph_cont = nullptr;
  s->graph_steps = 0;
}

bool fused_path(const ci_solver* s) { return s->opt.step_kernel == 3; }

int capture(ci_solver* s, cudaGraphExec_t* out, int steps, bool first) {
  cudaGraph_t g = nullptr;
  CI_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  if (fused_path(s))
    err = enqueue_fused(s, steps, first, false);
  else
    for (int i = 0; i < steps && err == cudaSuccess; i++) err = enqueue_step(s, false);
  cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
  if (err != cudaSuccess) return fail(CI_ERR_CUDA, "graph capture: %s", cudaGetErrorString(err));
  if (e2 != cudaSuccess) return fail(CI_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e2));
  err = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (err != cudaSuccess) return fail(CI_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(err));
  return CI_OK;
}

// Fused path: `graph` runs G steps from a complete state, `graph_cont` G steps that
// continue a previous block; neither completes the nodes at its end, so blocks chain
// and one k_finalize_nodes closes the call.  Two-kernel path: `graph` only.
int build_graph(ci_solver* s, int steps) {
  destroy_graph(s);
  int rc = capture(s, &s->graph, steps, true);
  if (!rc && fused_path(s)) rc = capture(s, &s->graph_cont, steps, false);
  if (rc) {
    destroy_graph(s);
    return rc;
  }
  s->graph_steps = steps;
  return CI_OK;
}

template <typename T>
int upload(DBuf<T>& b, const std::vector<T>& h, cudaStream_t st);

// Task kernel (step_kernel = 2): one descriptor per (task kind, position in the task
// order of the chunks) -- the chunk's ChunkInfo, its id, the length of its dependency
// list and the list (the chunks owning one of its local nodes for the element task, the
// chunks holding a local entry of a node it owns for the node task) in a fixed stride,
// so that a CTA copies the next task's descriptor into shared memory in one round trip;
// record buffers, counters and the number of CTAs kept resident.
int setup_flow(ci_solver* s) {
  const ci::Plan& P = s->plan;
  const int C = s->C;
  std::vector<int> own_row, own_idx, touch_row, touch_idx;
  const int longest = ci::flow_lists(P, &own_row, &own_idx, &touch_row, &touch_idx);
  const std::vector<int> order = ci::flow_order(C, own_row, own_idx);
  if ((int)order.size() != C) return fail(CI_ERR_INVALID, "task order of %d chunks has %zu", C, order.size());
  const int stride = ci::kFlowDescHead + ((longest + 3) & ~3);
  std::vector<int> desc(2 * (size_t)C * stride, 0);
  for (int kind = 0; kind < 2; kind++)
    for (int r = 0; r < C; r++) {
      const int c = order[r];
      int* d = desc.data() + ((size_t)kind * C + r) * stride;
      std::memcpy(d, &P.chunks[c], sizeof(ci::ChunkInfo));
      const std::vector<int>& row = kind == 0 ? own_row : touch_row;
      const std::vector<int>& idx = kind == 0 ? own_idx : touch_idx;
      d[ci::kFlowDescChunk] = c;
      d[ci::kFlowDescCount] = row[c + 1] - row[c];
      std::copy(idx.begin() + row[c], idx.begin() + row[c + 1], d + ci::kFlowDescHead);
    }
  s->flow_stride = stride;
  s->flow_smem = s->smem_bytes + 2 * sizeof(int) * (size_t)stride;
  int rc;
  if ((rc = upload(s->d_flow_desc, desc, s->stream))) return rc;
  CI_CUDA(s->d_rec.alloc(3 * (size_t)s->N));
  {
    // the records go from a node task to the element tasks of the same step: keep them
    // in L2 (a persisting access window over the one allocation).  Best effort: where the
    // device or its partitioning offers no persisting L2, the solver runs without it.
    int max_persist = 0, max_window = 0;
    const size_t bytes = sizeof(float4) * 3 * (size_t)s->N;
    bool ok = cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, s->device) ==
                  cudaSuccess &&
              cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, s->device) ==
                  cudaSuccess &&
              max_persist > 0 && max_window > 0;
    if (ok) {
      const size_t limit = std::min(bytes, (size_t)max_persist);
      cudaStreamAttrValue attr = {};
      attr.accessPolicyWindow.base_ptr = s->d_rec.p;
      attr.accessPolicyWindow.num_bytes = std::min(bytes, (size_t)max_window);
      attr.accessPolicyWindow.hitRatio =
          (float)std::min(1.0, (double)limit / (double)attr.accessPolicyWindow.num_bytes);
      attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
      attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
      ok = cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, limit) == cudaSuccess &&
           cudaStreamSetAttribute(s->stream, cudaStreamAttributeAccessPolicyWindow, &attr) ==
               cudaSuccess;
    }
    if (!ok) cudaGetLastError();  // not an error of the solver's: clear it
  }
  CI_CUDA(s->d_flow_ctr.alloc(2 * (size_t)C + 2));
  auto kern = s->opt.mode != CI_MODE_REFCOMPAT ? ci::k_flow_qp10<ci::EM_J2, 128>
                                               : ci::k_flow_qp10<ci::EM_REFCOMPAT, 128>;
  CI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->flow_smem));
  int per_sm = 0, sms = 0;
  CI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, s->flow_smem));
  CI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
  s->flow_ctas = std::max(1, std::min(per_sm * sms, C));
  return CI_OK;
}

// n steps in launches of the task kernel (at most kFlowMaxSteps steps each, and few
// enough that the task count C (2 k + 1) fits an int), each from a complete state in
// buffer A to a complete state in A.
constexpr int kFlowMaxSteps = 1 << 16;

cudaError_t enqueue_flow(ci_solver* s, int n) {
  const int C = s->C;
  const ci::ElemParams ep = s->elem_params((float)s->dt, true);
  const ci::NodeParams np = s->node_params();
  for (int done = 0; done < n;) {
    const int k = std::min({n - done, kFlowMaxSteps, (INT_MAX - C) / (2 * C)});
    ci::FlowArgs F;
    F.A[0] = s->fused_args(true, 0, false, false);
    F.A[1] = s->fused_args(false, 1, false, false);
    for (int p = 0; p < 2; p++) {
      F.rec_a[p] = s->d_rec.p + (size_t)p * s->N;
      F.rec_b[p] = reinterpret_cast<float2*>(s->d_rec.p + 2 * (size_t)s->N) + (size_t)p * s->N;
    }
    F.desc = s->d_flow_desc.p;
    F.desc_stride = s->flow_stride;
    F.node_done = s->d_flow_ctr.p;
    F.elem_done = s->d_flow_ctr.p + C;
    F.task_ctr = s->d_flow_ctr.p + 2 * C;
    F.abort_flag = s->d_flow_ctr.p + 2 * C + 1;
    F.C = C;
    F.nsteps = k;
    F.wait_ns = s->flow_wait_ns;
    F.stall_chunk = s->flow_stall_chunk;
    s->flow_stall_chunk = -1;
    s->flow_wait_ns = ci::kFlowWaitNs;
    cudaError_t e;
    // progress counters to -1, task counter and abort flag to 0
    if ((e = cudaMemsetAsync(s->d_flow_ctr.p, 0xff, sizeof(int) * 2 * (size_t)C, s->stream))) return e;
    if ((e = cudaMemsetAsync(F.task_ctr, 0, 2 * sizeof(int), s->stream))) return e;
    if (s->opt.mode != CI_MODE_REFCOMPAT)
      ci::k_flow_qp10<ci::EM_J2, 128><<<s->flow_ctas, 128, s->flow_smem, s->stream>>>(F, ep, np);
    else
      ci::k_flow_qp10<ci::EM_REFCOMPAT, 128><<<s->flow_ctas, 128, s->flow_smem, s->stream>>>(F, ep, np);
    if ((e = cudaGetLastError())) return e;
    if (k & 1) {
      const size_t b = sizeof(double) * 3 * (size_t)s->N;
      if ((e = cudaMemcpyAsync(s->d_u.p, s->d_ub.p, b, cudaMemcpyDeviceToDevice, s->stream))) return e;
      if ((e = cudaMemcpyAsync(s->d_v.p, s->d_vb.p, b, cudaMemcpyDeviceToDevice, s->stream))) return e;
    }
    done += k;
  }
  return cudaSuccess;
}

// Enqueue n steps; the last stores the acceleration for energy read-back.
int enqueue_steps(ci_solver* s, int n) {
  if (n <= 0) return CI_OK;
  if (s->opt.step_kernel == 2) {
    CI_CUDA(enqueue_flow(s, n));
    s->steps_done += n;
    return CI_OK;
  }
  if (fused_path(s)) {
    // chained graphs of G (even) steps, then the remainder directly and the completion
    const int G = (s->opt.graph_steps > 0 ? s->opt.graph_steps : 32) & ~1;
    int rest = n;
    bool chained = false;
    if (G >= 2 && rest > G) {
      if (!s->graph || !s->graph_cont || s->graph_steps != G) {
        const int rc = build_graph(s, G);
        if (rc) return rc;
      }
      while (rest > G) {
        CI_CUDA(cudaGraphLaunch(chained ? s->graph_cont : s->graph, s->stream));
        chained = true;
        rest -= G;
      }
    }
    CI_CUDA(enqueue_fused(s, rest, !chained, true));
    s->steps_done += n;
    return CI_OK;
  }
  const int G = s->opt.graph_steps > 0 ? s->opt.graph_steps : 32;
  int rest = n - 1;
  if (rest >= G) {
    if (!s->graph || s->graph_steps != G) {
      const int rc = build_graph(s, G);
      if (rc) return rc;
    }
    while (rest >= G) {
      CI_CUDA(cudaGraphLaunch(s->graph, s->stream));
      rest -= G;
    }
  }
  for (; rest > 0; rest--) CI_CUDA(enqueue_step(s, false));
  CI_CUDA(enqueue_step(s, true));
  s->steps_done += n;
  return CI_OK;
}

int require_started(ci_solver* s) {
  if (!s) return fail(CI_ERR_INVALID, "null solver");
  if (!s->started) return fail(CI_ERR_INVALID, "call ci_start or ci_solve before stepping");
  return CI_OK;
}

template <typename T>
int upload(DBuf<T>& b, const std::vector<T>& h, cudaStream_t st) {
  CI_CUDA(b.alloc(h.size()));
  if (!h.empty())
    CI_CUDA(cudaMemcpyAsync(b.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
  return CI_OK;
}

}  // namespace

// ---- binary state file (restart, parity dumps) ----
// Layout (little-endian, as written by this library): StateHeader, then X [3N] and
// vel0 [3] (double, caller order), u, v [3][N] (double, plan order), mass [N] (float),
// contact [N] (u8), sigma_a [E*nq] (float4), sigma_b [E*nq] (float2), epbar [E*nq]
// (float), chunk work sums [4C] (double).  The plan order is a function of the mesh and
// the chunk options, which the header records and ci_load_state checks.
namespace {
struct StateHeader {
  char magic[8];
  int32_t version, N, E, npe, nq, C, mode, lumping, chunk_elements, chunk_nodes, started;
  int64_t S, Lt, steps_done;
  double dt;
};
const char kStateMagic[8] = {'C', 'I', 'G', 'B', 'S', 'T', 'A', 'T'};

template <typename T>
int dev_to_file(FILE* f, const T* d, size_t n, cudaStream_t st) {
  std::vector<T> h(n);
  if (n) {
    CI_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    CI_CUDA(cudaStreamSynchronize(st));
  }
  if (n && fwrite(h.data(), sizeof(T), n, f) != n) return fail(CI_ERR_IO, "state file: write failed");
  return CI_OK;
}

template <typename T>
int file_to_dev(FILE* f, T* d, size_t n, cudaStream_t st) {
  std::vector<T> h(n);
  if (n && fread(h.data(), sizeof(T), n, f) != n) return fail(CI_ERR_IO, "state file: truncated");
  if (n) {
    CI_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(T) * n, cudaMemcpyHostToDevice, st));
    CI_CUDA(cudaStreamSynchronize(st));
  }
  return CI_OK;
}

struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) fclose(f);
  }
};
}  // namespace

namespace {
// x (caller AoS) = X + u (plan SoA), v likewise; one thread per caller node
// Shape-function gradients in reference coordinates, FP64 (the element geometry of
// Rule<NPE>: corners L = (xi, eta, 1-xi-eta-zeta, zeta), CalculiX edge order).
template <int NPE>
__device__ void ref_grad_f64(int q, double (&G)[NPE][3]) {
  const double dL[4][3] = {{1, 0, 0}, {0, 1, 0}, {-1, -1, -1}, {0, 0, 1}};
  if (NPE == 4) {
    for (int c = 0; c < 4; c++)
      for (int j = 0; j < 3; j++) G[c][j] = dL[c == 0 ? 2 : c == 1 ? 0 : c == 2 ? 1 : 3][j];
    return;
  }
  const double a = 0.58541019662496845446, b = 0.13819660112501051518;
  const double L[4] = {q == 1 ? a : b, q == 2 ? a : b, q == 0 ? a : b, q == 3 ? a : b};
  const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
  for (int c = 0; c < 4; c++)
    for (int j = 0; j < 3; j++) G[c][j] = (4 * L[c] - 1) * dL[c][j];
  for (int k = 0; k < 6 && 4 + k < NPE; k++)
    for (int j = 0; j < 3; j++)
      G[4 + k][j] = 4 * (L[ea[k]] * dL[eb[k]][j] + L[eb[k]] * dL[ea[k]][j]);
}

// Deformation gradient F = I + du/dX at every Gauss point, FP64, plan order [E][nq][9]
// (row a, column j: delta_aj + d u_a / d X_j); one CTA per chunk.
template <int NPE>
__global__ void __launch_bounds__(128) k_defgrad(ci::DevPlan P, const double* u0, const double* u1,
                                                 const double* u2, int nq, double* F) {
  const ci::ChunkInfo ch = P.chunks[blockIdx.x];
  const int ne = ch.elem_end - ch.elem_begin;
  const double* uk[3] = {u0, u1, u2};
  for (int idx = threadIdx.x; idx < ne * nq; idx += blockDim.x) {
    const int e = ch.elem_begin + idx / nq, q = idx % nq;
    double G[NPE][3];
    ref_grad_f64<NPE>(q, G);
    double J0[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Gu[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < NPE; i++) {
      const int l = P.conn_local[(size_t)i * P.E + e];
      const int lb = ch.local_begin + l;
      const int g = l < ch.n_own ? ch.own_begin + l : P.local_gid[lb];
      for (int k = 0; k < 3; k++) {
        const double X = P.local_x0[(size_t)k * P.Lt + lb], U = uk[k][g];
        for (int j = 0; j < 3; j++) {
          J0[3 * k + j] += X * G[i][j];
          Gu[3 * k + j] += U * G[i][j];
        }
      }
    }
    const double c00 = J0[4] * J0[8] - J0[5] * J0[7], c01 = J0[5] * J0[6] - J0[3] * J0[8],
                 c02 = J0[3] * J0[7] - J0[4] * J0[6];
    const double r = 1.0 / (J0[0] * c00 + J0[1] * c01 + J0[2] * c02);
    const double Ji[9] = {c00 * r, (J0[2] * J0[7] - J0[1] * J0[8]) * r,
                          (J0[1] * J0[5] - J0[2] * J0[4]) * r, c01 * r,
                          (J0[0] * J0[8] - J0[2] * J0[6]) * r, (J0[2] * J0[3] - J0[0] * J0[5]) * r,
                          c02 * r, (J0[1] * J0[6] - J0[0] * J0[7]) * r,
                          (J0[0] * J0[4] - J0[1] * J0[3]) * r};
    double* out = F + 9 * ((size_t)e * nq + q);
    for (int a = 0; a < 3; a++)
      for (int j = 0; j < 3; j++)
        out[3 * a + j] = (a == j ? 1.0 : 0.0) + Gu[3 * a + 0] * Ji[0 * 3 + j] +
                         Gu[3 * a + 1] * Ji[1 * 3 + j] + Gu[3 * a + 2] * Ji[2 * 3 + j];
  }
}

// Strain and stress output of the reference's update (include/dynamics_kernels.h:117-130,
// FEAnalysis::calculate_stress_strain, include/analysis.h:479-503), FP64, one thread per
// element, plan order [E][12]: at the parametric point (0, 0, 0) -- corner 2 of the
// element geometry, L = (0, 0, 1, 0) -- the Jacobian of the current positions X + u, the
// strain B u of the total displacement u in the reference's Voigt order (xx, yy, zz,
// gamma_xy, gamma_yz, gamma_xz; include/tetrahedral.h:442-484) and the stress D strain
// with the isotropic elastic D of include/tetrahedral.h:486-512.
template <int NPE>
__global__ void __launch_bounds__(128) k_elem_strain_stress(ci::DevPlan P, const double* u0,
                                                            const double* u1, const double* u2,
                                                            double E, double nu, double* out) {
  const ci::ChunkInfo ch = P.chunks[blockIdx.x];
  const double* uk[3] = {u0, u1, u2};
  // dN/dxi at L = (0, 0, 1, 0): tet4 corners are dL; tet10 corners (4 L_c - 1) dL_c and
  // edges 4 (L_a dL_b + L_b dL_a), nonzero only on the edges touching corner 2
  const double dL[4][3] = {{1, 0, 0}, {0, 1, 0}, {-1, -1, -1}, {0, 0, 1}};
  for (int e = ch.elem_begin + threadIdx.x; e < ch.elem_end; e += blockDim.x) {
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, uu[NPE][3], G[NPE][3];
    for (int i = 0; i < NPE; i++) {
      if (NPE == 4) {
        for (int j = 0; j < 3; j++) G[i][j] = dL[i][j];
      } else if (i < 4) {
        for (int j = 0; j < 3; j++) G[i][j] = (i == 2 ? 3.0 : -1.0) * dL[i][j];
      } else {
        // edge order 4:(0,1) 5:(1,2) 6:(2,0) 7:(0,3) 8:(1,3) 9:(2,3); L_2 = 1, others 0
        const int other = i == 5 ? 1 : i == 6 ? 0 : i == 9 ? 3 : -1;
        for (int j = 0; j < 3; j++) G[i][j] = other < 0 ? 0.0 : 4.0 * dL[other][j];
      }
      const int l = P.conn_local[(size_t)i * P.E + e];
      const int lb = ch.local_begin + l;
      const int g = l < ch.n_own ? ch.own_begin + l : P.local_gid[lb];
      for (int k = 0; k < 3; k++) {
        uu[i][k] = uk[k][g];
        const double x = (double)P.local_x0[(size_t)k * P.Lt + lb] + uu[i][k];
        for (int j = 0; j < 3; j++) J[3 * k + j] += x * G[i][j];
      }
    }
    const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8],
                 c02 = J[3] * J[7] - J[4] * J[6];
    const double r = 1.0 / (J[0] * c00 + J[1] * c01 + J[2] * c02);
    const double Ji[9] = {c00 * r, (J[2] * J[7] - J[1] * J[8]) * r, (J[1] * J[5] - J[2] * J[4]) * r,
                          c01 * r, (J[0] * J[8] - J[2] * J[6]) * r, (J[2] * J[3] - J[0] * J[5]) * r,
                          c02 * r, (J[1] * J[6] - J[0] * J[7]) * r, (J[0] * J[4] - J[1] * J[3]) * r};
    double L[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // L[a][b] = sum_i u_ia dN_i/dx_b
    for (int i = 0; i < NPE; i++)
      for (int b = 0; b < 3; b++) {
        const double dn = Ji[0 * 3 + b] * G[i][0] + Ji[1 * 3 + b] * G[i][1] + Ji[2 * 3 + b] * G[i][2];
        for (int a = 0; a < 3; a++) L[3 * a + b] += uu[i][a] * dn;
      }
    const double eps[6] = {L[0], L[4], L[8], L[1] + L[3], L[5] + L[7], L[2] + L[6]};
    const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double* o = out + 12 * (size_t)e;
    for (int k = 0; k < 6; k++) o[k] = eps[k];
    for (int k = 0; k < 3; k++)
      o[6 + k] = c * ((1.0 - nu) * eps[k] + nu * (eps[(k + 1) % 3] + eps[(k + 2) % 3]));
    for (int k = 3; k < 6; k++) o[6 + k] = c * 0.5 * (1.0 - 2.0 * nu) * eps[k];
  }
}

__global__ void k_state_to_caller(const double* u, const double* v, const double* Xc,
                                  const int* node_new, int N, double* xc, double* vc) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int i = node_new[n];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (xc) xc[3 * (size_t)n + k] = Xc[3 * (size_t)n + k] + u[(size_t)k * N + i];
    if (vc) vc[3 * (size_t)n + k] = v[(size_t)k * N + i];
  }
}

__global__ void k_state_from_caller(const double* xc, const double* vc, const double* Xc,
                                    const int* node_new, int N, double* u, double* v) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int i = node_new[n];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    u[(size_t)k * N + i] = xc[3 * (size_t)n + k] - Xc[3 * (size_t)n + k];
    v[(size_t)k * N + i] = vc[3 * (size_t)n + k];
  }
}

// The caller-order exchange buffers; X is uploaded again after it changes
// (ci_initialize, ci_load_state).
int ensure_exchange(ci_solver* s) {
  const size_t n3 = 3 * (size_t)s->N;
  if (!s->d_xc.p) {
    CI_CUDA(s->d_xc.alloc(n3));
    CI_CUDA(s->d_vc.alloc(n3));
    CI_CUDA(s->d_Xc.alloc(n3));
    CI_CUDA(s->d_node_new.alloc(s->N));
    CI_CUDA(cudaMemcpyAsync(s->d_node_new.p, s->plan.node_new.data(), sizeof(int) * s->N,
                            cudaMemcpyHostToDevice, s->stream));
  }
  if (s->xc_stale) {
    CI_CUDA(cudaMemcpyAsync(s->d_Xc.p, s->X.data(), sizeof(double) * n3, cudaMemcpyHostToDevice,
                            s->stream));
    s->xc_stale = false;
  }
  return CI_OK;
}
}  // namespace

extern "C" {

int ci_abi_version(void) { return CI_ABI_VERSION; }

const char* ci_last_error(void) { return g_last_error.c_str(); }

void ci_default_options(ci_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->mode = CI_MODE_J2;
  o->lumping = CI_LUMP_HRZ;
  o->gravity[2] = -9.81;
}

int ci_create(const ci_mesh* mesh, const ci_material* mat, const ci_wall* wall,
              const ci_options* opt, ci_solver** out) {
  if (!mesh || !mat || !wall || !out) return fail(CI_ERR_INVALID, "null argument");
  *out = nullptr;
  if (mesh->nodes_per_element != 4 && mesh->nodes_per_element != 10)
    return fail(CI_ERR_UNSUPPORTED, "nodes_per_element must be 4 or 10");
  if (!mesh->xloc || !mesh->element_nodes || mesh->num_nodes <= 0 || mesh->num_elements <= 0)
    return fail(CI_ERR_INVALID, "empty mesh");
  if (mat->beta != 0.0) return fail(CI_ERR_UNSUPPORTED, "only isotropic hardening (beta = 0)");
  if (!(mat->E > 0.0) || !(mat->rho > 0.0) || !(mat->nu > -1.0 && mat->nu < 0.5))
    return fail(CI_ERR_INVALID, "material needs E > 0, rho > 0, -1 < nu < 0.5");
  std::unique_ptr<ci_solver> s(new ci_solver());
  if (opt)
    s->opt = *opt;
  else
    ci_default_options(&s->opt);
  if (s->opt.mode != CI_MODE_J2 && s->opt.mode != CI_MODE_REFCOMPAT)
    return fail(CI_ERR_INVALID, "unknown mode");
  if (s->opt.step_kernel < 0 || s->opt.step_kernel > 3)
    return fail(CI_ERR_INVALID, "unknown step_kernel");
  if (s->opt.block_threads == 0) s->opt.block_threads = 128;
  if (s->opt.elem_lanes == 0) s->opt.elem_lanes = 4;
  if (s->opt.step_kernel == 2 &&
      (mesh->nodes_per_element != 10 || s->opt.elem_lanes != 4 || s->opt.block_threads != 128))
    return fail(CI_ERR_UNSUPPORTED,
                "step_kernel 2 (task kernel) needs tet10, elem_lanes 4 and block_threads 128");
  if (s->opt.elem_lanes != 1 && s->opt.elem_lanes != 4)
    return fail(CI_ERR_INVALID, "elem_lanes must be 1 or 4");
  if (s->opt.block_threads != 64 && s->opt.block_threads != 128 && s->opt.block_threads != 256)
    return fail(CI_ERR_INVALID, "block_threads must be 64, 128 or 256");
  s->mat = *mat;
  s->wall = *wall;
  s->N = mesh->num_nodes;
  s->E = mesh->num_elements;
  s->npe = mesh->nodes_per_element;
  s->nq = s->npe == 4 ? 1 : 4;
  s->device = s->opt.device;
  CI_CUDA(cudaSetDevice(s->device));
  int smem_max = 0;
  CI_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
  // the plan and the sizes that follow from it (built again below with the task kernel's
  // chunk budget when that kernel runs and the budget is automatic)
  auto make_plan = [&](int chunk_nodes) -> int {
    std::string err;
    if (!ci::build_plan(s->N, s->E, s->npe, mesh->xloc, mesh->element_nodes,
                        s->opt.chunk_elements, chunk_nodes, ci::kDefaultTargetCtas, &s->plan, &err))
      return fail(CI_ERR_INVALID, "%s", err.c_str());
    s->C = s->plan.n_chunks;
    s->S = s->plan.slot_row[s->N];
    s->Lt = (long long)s->plan.local_gid.size();
    // fused kernels: 40 B per local node (+ alignment); the element kernel: 36 B
    s->smem_bytes = 40 * ((size_t)s->plan.max_local + 2);
    if ((long long)s->smem_bytes + 1024 > smem_max)
      return fail(CI_ERR_TOO_LARGE, "chunk needs %zu B of shared memory", s->smem_bytes);
    return CI_OK;
  };
  int rc;
  if ((rc = make_plan(s->opt.chunk_nodes))) return rc;
  s->X0.assign(mesh->xloc, mesh->xloc + 3 * (size_t)s->N);
  s->X = s->X0;
  s->vel0.assign(3, 0.0);

  CI_CUDA(s->npe == 4 ? configure_npe<4>((int)s->smem_bytes) : configure_npe<10>((int)s->smem_bytes));
  if (s->opt.step_kernel == 0) {
    // automatic: the task kernel when the chunks of a four-lane tet10 mesh need more than
    // 0.8 of a round of the fused kernel's resident CTAs -- meshes whose chunks are cut by
    // the local-node budget -- else the fused kernel (measured: the 604,800-element shell,
    // 1.9 rounds, 98.0 against 121.9 us per step; half of it, 0.95 rounds, 58.1 against
    // 63.4; the quad cube, 0.66 rounds of small chunks, 19.4 against 14.9).
    s->opt.step_kernel = 3;
    if (s->npe == 10 && s->opt.elem_lanes == 4 && s->opt.block_threads == 128) {
      int per_sm = 0, sms = 0;
      CI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, ci::k_step_qp10<ci::EM_J2, 128>, 128, s->smem_bytes));
      CI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
      if (5LL * s->C > 4LL * per_sm * sms) s->opt.step_kernel = 2;
    }
  }
  if (s->opt.step_kernel == 2 && s->opt.chunk_nodes == 0) {
    // smaller chunks for the task kernel: six 768-node tiles per SM leave the SM a larger
    // L1 for the read-only connectivity and index loads (shell: 98 against 107 us per
    // step with the 896-node default, which suits the fused kernel)
    if ((rc = make_plan(kTaskChunkNodes))) return rc;
    CI_CUDA(configure_npe<10>((int)s->smem_bytes));
  }
  const ci::Plan& P = s->plan;
  CI_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  CI_CUDA(cudaEventCreate(&s->ev0));
  CI_CUDA(cudaEventCreate(&s->ev1));
  if ((rc = upload(s->d_chunks, P.chunks, s->stream))) return rc;
  if ((rc = upload(s->d_conn, P.conn_local, s->stream))) return rc;
  if ((rc = upload(s->d_color, P.color, s->stream))) return rc;
  if ((rc = upload(s->d_lgid, P.local_gid, s->stream))) return rc;
  if ((rc = upload(s->d_lslot, P.local_slot, s->stream))) return rc;
  if ((rc = upload(s->d_lsrow, P.local_srow, s->stream))) return rc;
  if ((rc = upload(s->d_slot_row, P.slot_row, s->stream))) return rc;
  const size_t N = s->N, E = s->E;
  CI_CUDA(s->d_lx0.alloc(3 * (size_t)s->Lt));
  CI_CUDA(s->d_u.alloc(3 * N));
  CI_CUDA(s->d_v.alloc(3 * N));
  CI_CUDA(s->d_slot.alloc(3 * (size_t)s->S));
  if (s->opt.step_kernel == 3 || s->opt.step_kernel == 2) {
    CI_CUDA(s->d_ub.alloc(3 * N));
    CI_CUDA(s->d_vb.alloc(3 * N));
    CI_CUDA(s->d_halo1.alloc(3 * (size_t)s->S));
  }
  if (s->opt.step_kernel == 2 && (rc = setup_flow(s.get()))) return rc;
  CI_CUDA(s->d_mass.alloc(N));
  CI_CUDA(s->d_d0.alloc(N));
  CI_CUDA(s->d_d0f.alloc(N));
  CI_CUDA(s->d_contact.alloc(N));
  CI_CUDA(s->d_acc.alloc(3 * N));
  CI_CUDA(s->d_sig_a.alloc(E * s->nq));
  CI_CUDA(s->d_sig_b.alloc(E * s->nq));
  CI_CUDA(s->d_epbar.alloc(E * s->nq));
  CI_CUDA(s->d_work.alloc(4 * (size_t)s->C));
  CI_CUDA(s->d_status.alloc(1));
  CI_CUDA(s->d_epart.alloc(3 * ((N + 255) / 256)));
  if ((rc = upload_reference(s.get()))) return rc;
  if ((rc = reset_state(s.get()))) return rc;
  *out = s.release();
  return CI_OK;
}

int ci_destroy(ci_solver* s) {
  if (!s) return CI_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  destroy_graph(s);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  cudaStream_t st = s->stream;
  const bool persisted = s->d_rec.p != nullptr;
  delete s;
  if (st) cudaStreamDestroy(st);
  // lines the solver's access window kept in L2 return to normal use (the persisting
  // limit itself belongs to this process's context and ends with it)
  if (persisted) cudaCtxResetPersistingL2Cache();
  return CI_OK;
}

int ci_initialize(ci_solver* s, const double pos[3], const double vel[3]) {
  if (!s || !pos || !vel) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  for (int i = 0; i < s->N; i++)
    for (int k = 0; k < 3; k++) s->X[3 * (size_t)i + k] = s->X0[3 * (size_t)i + k] + pos[k];
  for (int k = 0; k < 3; k++) s->vel0[k] = vel[k];
  s->xc_stale = true;
  int rc = upload_reference(s);
  if (rc) return rc;
  return reset_state(s);
}

int ci_start(ci_solver* s, double dt) {
  if (!s) return fail(CI_ERR_INVALID, "null solver");
  if (!(dt > 0.0)) return fail(CI_ERR_INVALID, "dt must be positive");
  CI_CUDA(cudaSetDevice(s->device));
  int rc = reset_history(s);
  if (rc) return rc;
  s->dt = dt;
  destroy_graph(s);
  if ((rc = compute_mass(s))) return rc;
  ci::k_node_init<false><<<(s->N + 255) / 256, 256, 0, s->stream>>>(
      s->node_arrays(), s->node_params(), nullptr, nullptr, s->d_d0f.p);
  CI_CUDA(cudaGetLastError());
  s->started = true;
  return check_status(s);
}

int ci_step(ci_solver* s, int nsteps) {
  int rc = require_started(s);
  if (rc) return rc;
  if (nsteps < 0) return fail(CI_ERR_INVALID, "nsteps < 0");
  CI_CUDA(cudaSetDevice(s->device));
  if ((rc = enqueue_steps(s, nsteps))) return rc;
  return check_status(s);
}

int ci_solve(ci_solver* s, double dt, double time_end, int export_interval) {
  (void)export_interval;
  int rc = ci_start(s, dt);
  if (rc) return rc;
  long long n = 0;
  for (double t = 0.0; t <= time_end; t += dt) n++;  // the reference's loop count
  while (n > 0) {
    const int chunk = (int)std::min<long long>(n, 1 << 20);
    if ((rc = ci_step(s, chunk))) return rc;
    n -= chunk;
  }
  return CI_OK;
}

int ci_steps_done(const ci_solver* s, long long* nsteps) {
  if (!s || !nsteps) return fail(CI_ERR_INVALID, "null argument");
  *nsteps = s->steps_done;
  return CI_OK;
}

int ci_get_state(ci_solver* s, double* x, double* v, double* mass, float* sigma, float* epbar,
                 unsigned char* contact) {
  if (!s) return fail(CI_ERR_INVALID, "null solver");
  CI_CUDA(cudaSetDevice(s->device));
  const int N = s->N, E = s->E, nq = s->nq;
  const ci::Plan& P = s->plan;
  if (x || v) {
    // permuted to the caller's order on the GPU, then one copy per array
    int rc = ensure_exchange(s);
    if (rc) return rc;
    k_state_to_caller<<<(N + 255) / 256, 256, 0, s->stream>>>(
        s->d_u.p, s->d_v.p, s->d_Xc.p, s->d_node_new.p, N, x ? s->d_xc.p : nullptr,
        v ? s->d_vc.p : nullptr);
    CI_CUDA(cudaGetLastError());
    if (x)
      CI_CUDA(cudaMemcpyAsync(x, s->d_xc.p, sizeof(double) * 3 * (size_t)N, cudaMemcpyDeviceToHost,
                              s->stream));
    if (v)
      CI_CUDA(cudaMemcpyAsync(v, s->d_vc.p, sizeof(double) * 3 * (size_t)N, cudaMemcpyDeviceToHost,
                              s->stream));
  }
  std::vector<float> hm, hep;
  std::vector<float4> hsa;
  std::vector<float2> hsb;
  std::vector<unsigned char> hc;
  if (mass) {
    hm.resize(N);
    CI_CUDA(cudaMemcpyAsync(hm.data(), s->d_mass.p, sizeof(float) * N, cudaMemcpyDeviceToHost,
                            s->stream));
  }
  if (sigma) {
    hsa.resize((size_t)E * nq);
    hsb.resize((size_t)E * nq);
    CI_CUDA(cudaMemcpyAsync(hsa.data(), s->d_sig_a.p, sizeof(float4) * hsa.size(),
                            cudaMemcpyDeviceToHost, s->stream));
    CI_CUDA(cudaMemcpyAsync(hsb.data(), s->d_sig_b.p, sizeof(float2) * hsb.size(),
                            cudaMemcpyDeviceToHost, s->stream));
  }
  if (epbar) {
    hep.resize((size_t)E * nq);
    CI_CUDA(cudaMemcpyAsync(hep.data(), s->d_epbar.p, sizeof(float) * hep.size(),
                            cudaMemcpyDeviceToHost, s->stream));
  }
  if (contact) {
    hc.resize(N);
    CI_CUDA(cudaMemcpyAsync(hc.data(), s->d_contact.p, N, cudaMemcpyDeviceToHost, s->stream));
  }
  CI_CUDA(cudaStreamSynchronize(s->stream));
  if (mass || contact)
    for (int i = 0; i < N; i++) {
      const int n = P.node_orig[i];
      if (mass) mass[n] = hm[i];
      if (contact) contact[n] = hc[i];
    }
  for (int pe = 0; pe < E; pe++) {
    const int oe = P.elem_orig[pe];
    for (int q = 0; q < nq; q++) {
      const size_t qi = (size_t)pe * nq + q, o = (size_t)oe * nq + q;
      if (sigma) {
        const float4 a = hsa[qi];
        const float2 b = hsb[qi];
        float* d = sigma + 6 * o;
        d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w; d[4] = b.x; d[5] = b.y;
      }
      if (epbar) epbar[o] = hep[qi];
    }
  }
  return CI_OK;
}

int ci_deformation_gradient(ci_solver* s, double* F) {
  if (!s || !F) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  const int E = s->E, nq = s->nq;
  const ci::Plan& P = s->plan;
  DBuf<double> d;
  CI_CUDA(d.alloc((size_t)9 * E * nq));
  const ci::DevPlan dp = s->dev_plan();
  if (s->npe == 4)
    k_defgrad<4><<<s->C, 128, 0, s->stream>>>(dp, s->d_u.p, s->d_u.p + s->N,
                                               s->d_u.p + 2 * (size_t)s->N, nq, d.p);
  else
    k_defgrad<10><<<s->C, 128, 0, s->stream>>>(dp, s->d_u.p, s->d_u.p + s->N,
                                                s->d_u.p + 2 * (size_t)s->N, nq, d.p);
  CI_CUDA(cudaGetLastError());
  std::vector<double> h((size_t)9 * E * nq);
  CI_CUDA(cudaMemcpyAsync(h.data(), d.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost,
                          s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  for (int pe = 0; pe < E; pe++)
    std::memcpy(F + (size_t)9 * nq * P.elem_orig[pe], h.data() + (size_t)9 * nq * pe,
                sizeof(double) * 9 * nq);
  return CI_OK;
}

int ci_get_nodal_fields(ci_solver* s, double* acc, double* strain, double* stress) {
  if (!s) return fail(CI_ERR_INVALID, "null solver");
  CI_CUDA(cudaSetDevice(s->device));
  const int N = s->N, E = s->E;
  const ci::Plan& P = s->plan;
  if (acc) {
    // the last step's acceleration, kept by the step that ends every ci_step call
    std::vector<float> a(3 * (size_t)N);
    CI_CUDA(cudaMemcpyAsync(a.data(), s->d_acc.p, sizeof(float) * a.size(), cudaMemcpyDeviceToHost,
                            s->stream));
    CI_CUDA(cudaStreamSynchronize(s->stream));
    for (int i = 0; i < N; i++)
      for (int k = 0; k < 3; k++)
        acc[3 * (size_t)P.node_orig[i] + k] = (double)a[(size_t)k * N + i];
  }
  if (!strain && !stress) return CI_OK;
  if (s->last_elem.empty()) {
    // for every node, the last element (caller order) that contains it: the reference
    // assigns element values to nodes in element order, so that element's value stays
    s->last_elem.assign(N, -1);
    for (int c = 0; c < s->C; c++) {
      const ci::ChunkInfo& ch = P.chunks[c];
      for (int e = ch.elem_begin; e < ch.elem_end; e++)
        for (int a = 0; a < s->npe; a++) {
          const int l = P.conn_local[(size_t)a * E + e];
          const int g = l < ch.n_own ? ch.own_begin + l : P.local_gid[ch.local_begin + l];
          int& le = s->last_elem[P.node_orig[g]];
          le = std::max(le, P.elem_orig[e]);
        }
    }
    s->elem_new.assign(E, 0);
    for (int e = 0; e < E; e++) s->elem_new[P.elem_orig[e]] = e;
  }
  DBuf<double> d;
  CI_CUDA(d.alloc((size_t)12 * E));
  const ci::DevPlan dp = s->dev_plan();
  if (s->npe == 4)
    k_elem_strain_stress<4><<<s->C, 128, 0, s->stream>>>(dp, s->d_u.p, s->d_u.p + N,
                                                          s->d_u.p + 2 * (size_t)N, s->mat.E,
                                                          s->mat.nu, d.p);
  else
    k_elem_strain_stress<10><<<s->C, 128, 0, s->stream>>>(dp, s->d_u.p, s->d_u.p + N,
                                                           s->d_u.p + 2 * (size_t)N, s->mat.E,
                                                           s->mat.nu, d.p);
  CI_CUDA(cudaGetLastError());
  std::vector<double> h((size_t)12 * E);
  CI_CUDA(cudaMemcpyAsync(h.data(), d.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost,
                          s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  for (int n = 0; n < N; n++) {
    const int le = s->last_elem[n];
    const double* src = le < 0 ? nullptr : h.data() + 12 * (size_t)s->elem_new[le];
    for (int k = 0; k < 6; k++) {
      if (strain) strain[6 * (size_t)n + k] = src ? src[k] : 0.0;
      if (stress) stress[6 * (size_t)n + k] = src ? src[6 + k] : 0.0;
    }
  }
  return CI_OK;
}

int ci_set_state(ci_solver* s, const double* x, const double* v) {
  if (!s || !x || !v) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  const int N = s->N;
  int rc = ensure_exchange(s);
  if (rc) return rc;
  CI_CUDA(cudaMemcpyAsync(s->d_xc.p, x, sizeof(double) * 3 * (size_t)N, cudaMemcpyHostToDevice,
                          s->stream));
  CI_CUDA(cudaMemcpyAsync(s->d_vc.p, v, sizeof(double) * 3 * (size_t)N, cudaMemcpyHostToDevice,
                          s->stream));
  k_state_from_caller<<<(N + 255) / 256, 256, 0, s->stream>>>(s->d_xc.p, s->d_vc.p, s->d_Xc.p,
                                                              s->d_node_new.p, N, s->d_u.p, s->d_v.p);
  CI_CUDA(cudaGetLastError());
  CI_CUDA(cudaStreamSynchronize(s->stream));
  return CI_OK;
}


int ci_save_state(ci_solver* s, const char* path) {
  if (!s || !path) return fail(CI_ERR_INVALID, "null argument");
  int rc = require_started(s);
  if (rc) return rc;
  CI_CUDA(cudaSetDevice(s->device));
  FILE* f = fopen(path, "wb");
  if (!f) return fail(CI_ERR_IO, "cannot open %s for writing", path);
  FileCloser fc{f};
  StateHeader h{};
  std::memcpy(h.magic, kStateMagic, 8);
  h.version = 1;
  h.N = s->N;
  h.E = s->E;
  h.npe = s->npe;
  h.nq = s->nq;
  h.C = s->C;
  h.mode = s->opt.mode;
  h.lumping = s->opt.lumping;
  h.chunk_elements = s->opt.chunk_elements;
  h.chunk_nodes = s->opt.chunk_nodes;
  h.started = 1;
  h.S = s->S;
  h.Lt = s->Lt;
  h.steps_done = s->steps_done;
  h.dt = s->dt;
  const size_t N = s->N, Q = (size_t)s->E * s->nq;
  if (fwrite(&h, sizeof(h), 1, f) != 1 || fwrite(s->X.data(), sizeof(double), 3 * N, f) != 3 * N ||
      fwrite(s->vel0.data(), sizeof(double), 3, f) != 3)
    return fail(CI_ERR_IO, "state file: write failed");
  if ((rc = dev_to_file(f, s->d_u.p, 3 * N, s->stream))) return rc;
  if ((rc = dev_to_file(f, s->d_v.p, 3 * N, s->stream))) return rc;
  if ((rc = dev_to_file(f, s->d_mass.p, N, s->stream))) return rc;
  if ((rc = dev_to_file(f, s->d_contact.p, N, s->stream))) return rc;
  if ((rc = dev_to_file(f, s->d_sig_a.p, Q, s->stream))) return rc;
  if ((rc = dev_to_file(f, s->d_sig_b.p, Q, s->stream))) return rc;
  if ((rc = dev_to_file(f, s->d_epbar.p, Q, s->stream))) return rc;
  if ((rc = dev_to_file(f, s->d_work.p, 4 * (size_t)s->C, s->stream))) return rc;
  return CI_OK;
}

int ci_load_state(ci_solver* s, const char* path) {
  if (!s || !path) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  FILE* f = fopen(path, "rb");
  if (!f) return fail(CI_ERR_IO, "cannot open %s", path);
  FileCloser fc{f};
  StateHeader h{};
  if (fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kStateMagic, 8) != 0 || h.version != 1)
    return fail(CI_ERR_IO, "%s is not a state file of this library", path);
  if (h.N != s->N || h.E != s->E || h.npe != s->npe || h.nq != s->nq || h.C != s->C ||
      h.S != s->S || h.Lt != s->Lt || h.mode != s->opt.mode || h.lumping != s->opt.lumping ||
      h.chunk_elements != s->opt.chunk_elements || h.chunk_nodes != s->opt.chunk_nodes)
    return fail(CI_ERR_INVALID, "state file was written for another mesh, plan or mode");
  if (!(h.dt > 0.0) || h.steps_done < 0) return fail(CI_ERR_IO, "state file: bad header");
  const size_t N = s->N, Q = (size_t)s->E * s->nq;
  std::vector<double> X(3 * N), vel0(3);
  if (fread(X.data(), sizeof(double), 3 * N, f) != 3 * N || fread(vel0.data(), sizeof(double), 3, f) != 3)
    return fail(CI_ERR_IO, "state file: truncated");
  s->X = X;
  s->vel0 = vel0;
  s->xc_stale = true;
  int rc = upload_reference(s);
  if (rc) return rc;
  destroy_graph(s);
  if ((rc = file_to_dev(f, s->d_u.p, 3 * N, s->stream))) return rc;
  if ((rc = file_to_dev(f, s->d_v.p, 3 * N, s->stream))) return rc;
  if ((rc = file_to_dev(f, s->d_mass.p, N, s->stream))) return rc;
  if ((rc = file_to_dev(f, s->d_contact.p, N, s->stream))) return rc;
  if ((rc = file_to_dev(f, s->d_sig_a.p, Q, s->stream))) return rc;
  if ((rc = file_to_dev(f, s->d_sig_b.p, Q, s->stream))) return rc;
  if ((rc = file_to_dev(f, s->d_epbar.p, Q, s->stream))) return rc;
  if ((rc = file_to_dev(f, s->d_work.p, 4 * (size_t)s->C, s->stream))) return rc;
  s->dt = h.dt;
  s->steps_done = h.steps_done;
  s->started = true;
  return CI_OK;
}

int ci_get_energy(ci_solver* s, ci_energy* e) {
  if (!s || !e) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  const int nb = (s->N + 255) / 256;
  ci::k_energy<<<nb, 256, 0, s->stream>>>(s->node_arrays(), s->node_params(), s->d_epart.p);
  CI_CUDA(cudaGetLastError());
  std::vector<double> part(3 * (size_t)nb), work(4 * (size_t)s->C);
  CI_CUDA(cudaMemcpyAsync(part.data(), s->d_epart.p, sizeof(double) * part.size(),
                          cudaMemcpyDeviceToHost, s->stream));
  CI_CUDA(cudaMemcpyAsync(work.data(), s->d_work.p, sizeof(double) * work.size(),
                          cudaMemcpyDeviceToHost, s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  double ke = 0, phi = 0, wg = 0, wi = 0, wp = 0;
  for (int b = 0; b < nb; b++) {
    ke += part[3 * b];
    phi += part[3 * b + 1];
    wg += part[3 * b + 2];
  }
  for (int c = 0; c < s->C; c++) {
    wi += work[4 * c];
    wp += work[4 * c + 1];
  }
  // initial kinetic energy and contact potential from the reference state
  double m_tot = 0.0, phi0 = 0.0;
  std::vector<float> hm(s->N);
  CI_CUDA(cudaMemcpy(hm.data(), s->d_mass.p, sizeof(float) * s->N, cudaMemcpyDeviceToHost));
  for (int i = 0; i < s->N; i++) {
    m_tot += hm[i];
    const int n = s->plan.node_orig[i];
    const double d = s->wall.normal[0] * s->X[3 * (size_t)n] + s->wall.normal[1] * s->X[3 * (size_t)n + 1] +
                     s->wall.normal[2] * s->X[3 * (size_t)n + 2] - s->wall.offset;
    if (d < 0.0) phi0 += 0.5 * s->wall.stiffness * d * d;
  }
  const double v2 = s->vel0[0] * s->vel0[0] + s->vel0[1] * s->vel0[1] + s->vel0[2] * s->vel0[2];
  e->kinetic = ke;
  e->internal = wi;
  e->plastic = wp;
  e->contact = -(phi - phi0);
  e->gravity = wg;
  e->kinetic0 = 0.5 * m_tot * v2;
  e->balance = ke + wi - e->contact - wg - e->kinetic0;
  return CI_OK;
}

int ci_get_status(ci_solver* s, unsigned int* status) {
  if (!s || !status) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  CI_CUDA(cudaMemcpyAsync(status, s->d_status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                          s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  return CI_OK;
}

int ci_internal_force(ci_solver* s, const double* x, const double* du, const float* sigma_in,
                      const float* epbar_in, double* f, float* sigma_out, float* epbar_out) {
  if (!s || !x || !du || !f) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  const int N = s->N, E = s->E, nq = s->nq;
  const ci::Plan& P = s->plan;
  std::vector<double> hu(3 * (size_t)N), hv(3 * (size_t)N);
  for (int i = 0; i < N; i++) {
    const int n = P.node_orig[i];
    for (int k = 0; k < 3; k++) {
      hu[(size_t)k * N + i] = x[3 * (size_t)n + k] - s->X[3 * (size_t)n + k];
      hv[(size_t)k * N + i] = du[3 * (size_t)n + k];
    }
  }
  CI_CUDA(s->d_u2.alloc(3 * (size_t)N));
  CI_CUDA(s->d_v2.alloc(3 * (size_t)N));
  CI_CUDA(s->d_f.alloc(3 * (size_t)N));
  CI_CUDA(cudaMemcpyAsync(s->d_u2.p, hu.data(), sizeof(double) * hu.size(), cudaMemcpyHostToDevice,
                          s->stream));
  CI_CUDA(cudaMemcpyAsync(s->d_v2.p, hv.data(), sizeof(double) * hv.size(), cudaMemcpyHostToDevice,
                          s->stream));
  const bool j2 = s->opt.mode == CI_MODE_J2;
  if (j2) {
    CI_CUDA(s->d_sig_a2.alloc((size_t)E * nq));
    CI_CUDA(s->d_sig_b2.alloc((size_t)E * nq));
    CI_CUDA(s->d_epbar2.alloc((size_t)E * nq));
    std::vector<float4> sa((size_t)E * nq, make_float4(0, 0, 0, 0));
    std::vector<float2> sb((size_t)E * nq, make_float2(0, 0));
    std::vector<float> ep((size_t)E * nq, 0.f);
    for (int pe = 0; pe < E; pe++)
      for (int q = 0; q < nq; q++) {
        const size_t qi = (size_t)pe * nq + q, o = (size_t)P.elem_orig[pe] * nq + q;
        if (sigma_in) {
          const float* d = sigma_in + 6 * o;
          sa[qi] = make_float4(d[0], d[1], d[2], d[3]);
          sb[qi] = make_float2(d[4], d[5]);
        }
        if (epbar_in) ep[qi] = epbar_in[o];
      }
    CI_CUDA(cudaMemcpyAsync(s->d_sig_a2.p, sa.data(), sizeof(float4) * sa.size(),
                            cudaMemcpyHostToDevice, s->stream));
    CI_CUDA(cudaMemcpyAsync(s->d_sig_b2.p, sb.data(), sizeof(float2) * sb.size(),
                            cudaMemcpyHostToDevice, s->stream));
    CI_CUDA(cudaMemcpyAsync(s->d_epbar2.p, ep.data(), sizeof(float) * ep.size(),
                            cudaMemcpyHostToDevice, s->stream));
  }
  ci::DevState D = s->dev_state(s->d_u2.p, s->d_v2.p);
  D.sig_a = s->d_sig_a2.p;
  D.sig_b = s->d_sig_b2.p;
  D.epbar = s->d_epbar2.p;
  CI_CUDA(launch_elem_mode(s, step_mode(s), D, s->elem_params(1.0f, false)));
  ci::k_force_sum<<<(N + 255) / 256, 256, 0, s->stream>>>(
      s->d_slot.p, s->d_slot.p + s->S, s->d_slot.p + 2 * s->S, s->d_slot_row.p, s->d_f.p, N);
  CI_CUDA(cudaGetLastError());
  std::vector<double> hf(3 * (size_t)N);
  CI_CUDA(cudaMemcpyAsync(hf.data(), s->d_f.p, sizeof(double) * hf.size(), cudaMemcpyDeviceToHost,
                          s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  for (int i = 0; i < N; i++)
    for (int k = 0; k < 3; k++) f[3 * (size_t)P.node_orig[i] + k] = hf[(size_t)k * N + i];
  if (j2 && (sigma_out || epbar_out)) {
    std::vector<float4> sa((size_t)E * nq);
    std::vector<float2> sb((size_t)E * nq);
    std::vector<float> ep((size_t)E * nq);
    CI_CUDA(cudaMemcpy(sa.data(), s->d_sig_a2.p, sizeof(float4) * sa.size(), cudaMemcpyDeviceToHost));
    CI_CUDA(cudaMemcpy(sb.data(), s->d_sig_b2.p, sizeof(float2) * sb.size(), cudaMemcpyDeviceToHost));
    CI_CUDA(cudaMemcpy(ep.data(), s->d_epbar2.p, sizeof(float) * ep.size(), cudaMemcpyDeviceToHost));
    for (int pe = 0; pe < E; pe++)
      for (int q = 0; q < nq; q++) {
        const size_t qi = (size_t)pe * nq + q, o = (size_t)P.elem_orig[pe] * nq + q;
        if (sigma_out) {
          float* d = sigma_out + 6 * o;
          d[0] = sa[qi].x; d[1] = sa[qi].y; d[2] = sa[qi].z; d[3] = sa[qi].w;
          d[4] = sb[qi].x; d[5] = sb[qi].y;
        }
        if (epbar_out) epbar_out[o] = ep[qi];
      }
  }
  return check_status(s);
}

int ci_lumped_mass(ci_solver* s, const double* x, double* mass) {
  if (!s || !x || !mass) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  const int N = s->N;
  const ci::Plan& P = s->plan;
  std::vector<double> hu(3 * (size_t)N);
  for (int i = 0; i < N; i++) {
    const int n = P.node_orig[i];
    for (int k = 0; k < 3; k++) hu[(size_t)k * N + i] = x[3 * (size_t)n + k] - s->X[3 * (size_t)n + k];
  }
  CI_CUDA(s->d_u2.alloc(3 * (size_t)N));
  CI_CUDA(s->d_v2.alloc(3 * (size_t)N));
  CI_CUDA(cudaMemcpyAsync(s->d_u2.p, hu.data(), sizeof(double) * hu.size(), cudaMemcpyHostToDevice,
                          s->stream));
  const ci::DevState D = s->dev_state(s->d_u2.p, s->d_v2.p);
  const int mode = s->opt.lumping == CI_LUMP_HRZ ? ci::EM_MASS_HRZ : ci::EM_MASS_ROWSUM;
  CI_CUDA(launch_elem_mode(s, mode, D, s->elem_params(0.f, false)));
  DBuf<float> m;
  CI_CUDA(m.alloc(N));
  ci::k_mass_sum<<<(N + 255) / 256, 256, 0, s->stream>>>(s->d_slot.p, s->d_slot_row.p, m.p, N);
  CI_CUDA(cudaGetLastError());
  std::vector<float> hm(N);
  CI_CUDA(cudaMemcpyAsync(hm.data(), m.p, sizeof(float) * N, cudaMemcpyDeviceToHost, s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  for (int i = 0; i < N; i++) mass[P.node_orig[i]] = hm[i];
  return check_status(s);
}

int ci_strain_energy(ci_solver* s, const double* u, double* energy, double* volume) {
  if (!s || !u || !energy || !volume) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  const int N = s->N;
  const ci::Plan& P = s->plan;
  std::vector<double> hv(3 * (size_t)N);
  for (int i = 0; i < N; i++)
    for (int k = 0; k < 3; k++) hv[(size_t)k * N + i] = u[3 * (size_t)P.node_orig[i] + k];
  CI_CUDA(s->d_u2.alloc(3 * (size_t)N));
  CI_CUDA(s->d_v2.alloc(3 * (size_t)N));
  CI_CUDA(cudaMemsetAsync(s->d_u2.p, 0, sizeof(double) * 3 * N, s->stream));
  CI_CUDA(cudaMemcpyAsync(s->d_v2.p, hv.data(), sizeof(double) * hv.size(), cudaMemcpyHostToDevice,
                          s->stream));
  DBuf<double> work;
  CI_CUDA(work.alloc(4 * (size_t)s->C));
  CI_CUDA(cudaMemsetAsync(work.p, 0, sizeof(double) * 4 * s->C, s->stream));
  ci::DevState D = s->dev_state(s->d_u2.p, s->d_v2.p);
  D.chunk_work = work.p;
  CI_CUDA(launch_elem_mode(s, ci::EM_REFCOMPAT, D, s->elem_params(1.0f, true)));
  std::vector<double> hw(4 * (size_t)s->C);
  CI_CUDA(cudaMemcpyAsync(hw.data(), work.p, sizeof(double) * hw.size(), cudaMemcpyDeviceToHost,
                          s->stream));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  double W = 0, V = 0;
  for (int c = 0; c < s->C; c++) {
    W += hw[4 * c];
    V += hw[4 * c + 2];
  }
  *energy = W;
  *volume = V;
  return check_status(s);
}

int ci_time_steps(ci_solver* s, int nsteps, float* ms) {
  int rc = require_started(s);
  if (rc) return rc;
  if (!ms) return fail(CI_ERR_INVALID, "null argument");
  CI_CUDA(cudaSetDevice(s->device));
  CI_CUDA(cudaStreamSynchronize(s->stream));
  CI_CUDA(cudaEventRecord(s->ev0, s->stream));
  if ((rc = enqueue_steps(s, nsteps))) return rc;
  CI_CUDA(cudaEventRecord(s->ev1, s->stream));
  CI_CUDA(cudaEventSynchronize(s->ev1));
  CI_CUDA(cudaEventElapsedTime(ms, s->ev0, s->ev1));
  return check_status(s);
}

int ci_time_kernels(ci_solver* s, int nsteps, float* out_ms) {
  int rc = require_started(s);
  if (rc) return rc;
  if (!out_ms || nsteps <= 0) return fail(CI_ERR_INVALID, "bad argument");
  CI_CUDA(cudaSetDevice(s->device));
  std::vector<cudaEvent_t> ev(3 * nsteps);
  for (auto& e : ev) CI_CUDA(cudaEventCreate(&e));
  double te = 0, tn = 0;
  if (s->opt.step_kernel == 2) {
    // one launch runs all the steps: out[0] = its duration per step, out[1] = 0
    CI_CUDA(cudaEventRecord(ev[0], s->stream));
    CI_CUDA(enqueue_flow(s, nsteps));
    CI_CUDA(cudaEventRecord(ev[1], s->stream));
    CI_CUDA(cudaEventSynchronize(ev[1]));
    float a;
    CI_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]));
    te = a;
  } else if (fused_path(s)) {
    // out[0]: mean k_step duration; out[1]: the end-of-call boundary finalise
    for (int i = 0; i < nsteps; i++) {
      const ci::FusedArgs F = s->fused_args((i & 1) == 0, i & 1, i == 0, false);
      CI_CUDA(cudaEventRecord(ev[3 * i], s->stream));
      CI_CUDA(launch_fused(s, F));
      CI_CUDA(cudaEventRecord(ev[3 * i + 1], s->stream));
    }
    const ci::FusedArgs F = s->fused_args((nsteps & 1) == 0, nsteps & 1, false, true);
    CI_CUDA(launch_finalize(s, F));
    CI_CUDA(cudaEventRecord(ev[2], s->stream));
    if (nsteps & 1) {
      const size_t b = sizeof(double) * 3 * (size_t)s->N;
      CI_CUDA(cudaMemcpyAsync(s->d_u.p, s->d_ub.p, b, cudaMemcpyDeviceToDevice, s->stream));
      CI_CUDA(cudaMemcpyAsync(s->d_v.p, s->d_vb.p, b, cudaMemcpyDeviceToDevice, s->stream));
    }
    CI_CUDA(cudaStreamSynchronize(s->stream));
    for (int i = 0; i < nsteps; i++) {
      float a;
      CI_CUDA(cudaEventElapsedTime(&a, ev[3 * i], ev[3 * i + 1]));
      te += a;
    }
    float b;
    CI_CUDA(cudaEventElapsedTime(&b, ev[3 * (nsteps - 1) + 1], ev[2]));
    tn = b;  // one finalise per call, spread over the call's steps below
  } else {
    const ci::DevState D = s->dev_state(s->d_u.p, s->d_v.p);
    const int nb = (s->N + 255) / 256;
    for (int i = 0; i < nsteps; i++) {
      CI_CUDA(cudaEventRecord(ev[3 * i], s->stream));
      CI_CUDA(launch_elem_mode(s, step_mode(s), D, s->elem_params((float)s->dt, true)));
      CI_CUDA(cudaEventRecord(ev[3 * i + 1], s->stream));
      ci::k_node<false, true><<<nb, 256, 0, s->stream>>>(s->node_arrays(), s->node_params());
      CI_CUDA(cudaGetLastError());
      CI_CUDA(cudaEventRecord(ev[3 * i + 2], s->stream));
    }
    CI_CUDA(cudaEventSynchronize(ev.back()));
    for (int i = 0; i < nsteps; i++) {
      float a, b;
      CI_CUDA(cudaEventElapsedTime(&a, ev[3 * i], ev[3 * i + 1]));
      CI_CUDA(cudaEventElapsedTime(&b, ev[3 * i + 1], ev[3 * i + 2]));
      te += a;
      tn += b;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  s->steps_done += nsteps;
  out_ms[0] = (float)(te / nsteps);
  out_ms[1] = (float)(tn / nsteps);
  return check_status(s);
}

int ci_step_kernel(const ci_solver* s) { return s ? s->opt.step_kernel : -1; }

int ci_debug_flow_stall(ci_solver* s, int chunk, double wait_seconds) {
  if (!s) return fail(CI_ERR_INVALID, "null solver");
  if (s->opt.step_kernel != 2) return fail(CI_ERR_UNSUPPORTED, "the solver does not run the task kernel");
  if (chunk < 0 || chunk >= s->C || !(wait_seconds > 0.0) || wait_seconds > 60.0)
    return fail(CI_ERR_INVALID, "bad chunk or wait");
  s->flow_stall_chunk = chunk;
  s->flow_wait_ns = (unsigned long long)(wait_seconds * 1e9);
  return CI_OK;
}

int ci_launches_per_step(const ci_solver* s) {
  // the task kernel launches once per call of any length (and per 65,536 steps)
  return s ? (s->opt.step_kernel == 1 ? 2 : 1) : 0;
}

int ci_plan_stats(const ci_mesh* mesh, int chunk_elements, int chunk_nodes, long long* stats,
                  int* perm_elems, int* perm_nodes) {
  if (!mesh || !stats) return fail(CI_ERR_INVALID, "null argument");
  ci::Plan P;
  std::string err;
  if (!ci::build_plan(mesh->num_nodes, mesh->num_elements, mesh->nodes_per_element, mesh->xloc,
                      mesh->element_nodes, chunk_elements, chunk_nodes, ci::kDefaultTargetCtas, &P, &err))
    return fail(CI_ERR_INVALID, "%s", err.c_str());
  stats[0] = P.n_chunks;
  stats[1] = P.max_colors;
  stats[2] = P.max_local;
  stats[3] = P.slot_row[P.N];
  stats[4] = P.max_chunk_elems;
  stats[5] = P.n_ghosts;
  stats[6] = P.n_boundary;
  std::vector<int> r0, i0, r1, i1;
  stats[7] = ci::flow_lists(P, &r0, &i0, &r1, &i1);
  if (perm_elems) std::memcpy(perm_elems, P.elem_orig.data(), sizeof(int) * P.E);
  if (perm_nodes) std::memcpy(perm_nodes, P.node_orig.data(), sizeof(int) * P.N);
  return CI_OK;
}

int ci_plan_verify(const ci_mesh* mesh, int chunk_elements, int chunk_nodes) {
  if (!mesh) return fail(CI_ERR_INVALID, "null argument");
  ci::Plan P;
  std::string err;
  if (!ci::build_plan(mesh->num_nodes, mesh->num_elements, mesh->nodes_per_element, mesh->xloc,
                      mesh->element_nodes, chunk_elements, chunk_nodes, ci::kDefaultTargetCtas, &P, &err))
    return fail(CI_ERR_INVALID, "%s", err.c_str());
  if (!ci::verify_plan(P, mesh->element_nodes, &err)) return fail(CI_ERR_INVALID, "%s", err.c_str());
  return CI_OK;
}

}  // extern "C"
