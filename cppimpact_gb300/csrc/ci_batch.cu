// ci_batch.cu -- many impact instances of uneven size advanced by one launch per step.
//
// Each instance (mesh, material, wall, initial state, its own dt and end time) is
// planned exactly as a single solve would plan it (ci_plan.cpp); the plans of all
// instances with the same element type are concatenated into one plan whose chunks
// carry their instance id.  The fused step kernel reads each chunk's parameters from
// per-instance tables and the global step from a device counter, so a captured graph
// of 32 steps can be replayed: an instance steps while step < nsteps, finalises its
// boundary nodes at step == nsteps and idles afterwards.  tet4 and tet10 groups run on
// two streams.  Because every instance runs the same kernels on the same plan as its
// single solve, its result is bitwise that of the unbatched run (tests check it).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cppimpact_gb300.h"
#include "ci_kernels.cuh"
#include "ci_plan.h"

namespace ci {
int set_last_error(int code, const char* msg);
}
using namespace ci;

namespace {

int fail(int code, const std::string& msg) { return ci::set_last_error(code, msg.c_str()); }

#define CB_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(CI_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
  } while (0)

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
    return count ? cudaMalloc(&p, sizeof(T) * count) : cudaSuccess;
  }
  template <typename V>
  cudaError_t upload(const std::vector<V>& h, cudaStream_t st) {
    cudaError_t e = alloc(h.size());
    if (e || h.empty()) return e;
    return cudaMemcpyAsync(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st);
  }
};

constexpr int kGraphSteps = 32;

struct Inst {
  int group = 0, index = 0;  // group (0 tet4, 1 tet10) and index within it
  int N = 0, E = 0, npe = 0;
  int node_off = 0, elem_off = 0;
  int nsteps = 0;
  double dt = 0.0;
  std::vector<double> X;        // reference positions (mesh + pos), caller order
  std::vector<int> node_orig;   // plan node -> caller node (instance-local)
  std::vector<int> elem_orig;   // plan element -> caller element (instance-local)
  ci_material mat;
  ci_wall wall;
  double vel[3];
};

struct Group {
  int npe = 0, nq = 0;
  int N = 0, E = 0, C = 0, n_bnd = 0;
  long long S = 0, Lt = 0;
  int max_local = 0;
  size_t smem = 0;
  int block_threads = 128, elem_lanes = 4, chunk_nodes = 896, chunk_elements = 0;
  float tuned_ms_per_step = 0.f;  // autotuner's trial time of the chosen shape (0: not tuned)
  std::vector<int> insts;  // global instance ids
  int max_steps = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  DBuf<ChunkInfo> chunks;
  DBuf<uint16_t> conn;
  DBuf<uint8_t> color;
  DBuf<int> lgid, lslot, lsrow, slot_row, bnd, node_inst;
  DBuf<float> lx0, slot0, slot1, mass, d0f, acc, epbar, peak;
  DBuf<double> ua, va, ub, vb, v0, d0, work;
  DBuf<unsigned char> contact;
  DBuf<float4> sig_a;
  DBuf<float2> sig_b;
  DBuf<unsigned int> status;
  DBuf<ElemParams> inst_ep;
  DBuf<NodeParams> inst_np;
  DBuf<int> inst_nsteps, step_ctr;
  ~Group() {
    if (graph) cudaGraphExecDestroy(graph);
    if (stream) cudaStreamDestroy(stream);
  }
};

}  // namespace

struct ci_batch {
  int device = 0;
  std::vector<Inst> inst;
  std::unique_ptr<Group> g[2];
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  bool done = false;
  ~ci_batch() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

namespace {

ElemParams make_ep(const ci_material& m, double dt) {
  ElemParams p{};
  p.dt = (float)dt;
  p.mu = (float)(m.E / (2.0 * (1.0 + m.nu)));
  p.lambda = (float)(m.E * m.nu / ((1.0 + m.nu) * (1.0 - 2.0 * m.nu)));
  const bool elastic = !(m.sigma_y0 > 0.0) || m.sigma_y0 > 1e30;
  p.sy0 = elastic ? 3.0e38f : (float)m.sigma_y0;
  p.H = (float)m.H;
  p.rho = (float)m.rho;
  p.accum_energy = 1;
  return p;
}

NodeParams make_np(const ci_wall& w, const double gravity[3], double dt, int N) {
  NodeParams p{};
  p.dt = dt;
  for (int k = 0; k < 3; k++) {
    p.g[k] = gravity[k];
    p.wall_n[k] = w.normal[k];
    p.gf[k] = (float)gravity[k];
    p.nf[k] = (float)w.normal[k];
  }
  p.wall_k = w.stiffness;
  p.N = N;
  return p;
}

FusedArgs group_args(const Group& G, int i_in_graph) {
  FusedArgs F{};
  F.P.chunks = G.chunks.p;
  F.P.conn_local = G.conn.p;
  F.P.color = G.color.p;
  F.P.local_gid = G.lgid.p;
  F.P.local_slot = G.lslot.p;
  F.P.local_srow = reinterpret_cast<const int2*>(G.lsrow.p);
  F.P.local_x0 = G.lx0.p;
  F.P.slot_row = G.slot_row.p;
  F.P.E = G.E;
  F.P.N = G.N;
  F.P.Lt = (int)G.Lt;
  const bool even = (i_in_graph & 1) == 0;
  const size_t N = G.N, S = G.S;
  for (int k = 0; k < 3; k++) {
    F.u_cur[k] = (even ? G.ua.p : G.ub.p) + k * N;
    F.v_cur[k] = (even ? G.va.p : G.vb.p) + k * N;
    F.u_prv[k] = (even ? G.ub.p : G.ua.p) + k * N;
    F.v_prv[k] = (even ? G.vb.p : G.va.p) + k * N;
    F.halo_cur[k] = (even ? G.slot0.p : G.slot1.p) + k * S;
    F.halo_prv[k] = (even ? G.slot1.p : G.slot0.p) + k * S;
    F.acc[k] = G.acc.p + k * N;
  }
  F.mass = G.mass.p;
  F.d0 = G.d0.p;
  F.d0f = G.d0f.p;
  F.contact = G.contact.p;
  F.sig_a = G.sig_a.p;
  F.sig_b = G.sig_b.p;
  F.epbar = G.epbar.p;
  F.chunk_work = G.work.p;
  F.status = G.status.p;
  F.state_final = 0;
  F.store_acc = 0;
  F.inst_ep = G.inst_ep.p;
  F.inst_np = G.inst_np.p;
  F.inst_nsteps = G.inst_nsteps.p;
  F.step_ctr = G.step_ctr.p;
  F.step_off = i_in_graph;
  return F;
}

template <int NPE, int BS>
cudaError_t launch_batch_bs(Group& G, const FusedArgs& F) {
  const ElemParams ep{};
  const NodeParams np{};
  if (NPE == 10 && G.elem_lanes == 4)
    k_step_qp10<EM_J2, BS, true><<<G.C, BS, G.smem, G.stream>>>(F, ep, np);
  else if (NPE == 10)
    k_step_t10<EM_J2, BS, true><<<G.C, BS, G.smem, G.stream>>>(F, ep, np);
  else
    k_step<NPE, EM_J2, BS, true><<<G.C, BS, G.smem, G.stream>>>(F, ep, np);
  return cudaGetLastError();
}

template <int NPE>
cudaError_t launch_batch(Group& G, const FusedArgs& F) {
  if (G.block_threads == 64) return launch_batch_bs<NPE, 64>(G, F);
  if (G.block_threads == 256) return launch_batch_bs<NPE, 256>(G, F);
  return launch_batch_bs<NPE, 128>(G, F);
}

template <int NPE, int BS>
cudaError_t configure_bs(int bytes) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_step<NPE, EM_J2, BS, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
    return e;
  if (NPE == 10) {
    if ((e = cudaFuncSetAttribute(k_step_qp10<EM_J2, BS, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
      return e;
    if ((e = cudaFuncSetAttribute(k_step_t10<EM_J2, BS, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
      return e;
  }
  return cudaFuncSetAttribute(k_elem<NPE, EM_MASS_HRZ, 256>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int NPE>
cudaError_t configure(int bytes) {
  cudaError_t e;
  if ((e = configure_bs<NPE, 64>(bytes))) return e;
  if ((e = configure_bs<NPE, 128>(bytes))) return e;
  if ((e = configure_bs<NPE, 256>(bytes))) return e;
  return cudaFuncSetAttribute(k_elem<NPE, EM_MASS_ROWSUM, 256>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// Build one element-type group from its instances.
int build_group(ci_batch* b, Group& G, const ci_instance* in, const ci_options& opt) {
  // Instances that pass the same mesh arrays share one plan (a parameter sweep over
  // one mesh plans it once); distinct meshes are planned on the host's cores.
  const size_t n_inst = G.insts.size();
  std::vector<size_t> src(n_inst), uniq;
  for (size_t j = 0; j < n_inst; j++) {
    const ci_mesh& a = in[G.insts[j]].mesh;
    src[j] = j;
    for (size_t u : uniq) {
      const ci_mesh& m = in[G.insts[u]].mesh;
      if (m.xloc == a.xloc && m.element_nodes == a.element_nodes && m.num_nodes == a.num_nodes &&
          m.num_elements == a.num_elements && m.nodes_per_element == a.nodes_per_element) {
        src[j] = u;
        break;
      }
    }
    if (src[j] == j) uniq.push_back(j);
  }
  std::vector<Plan> built(n_inst);
  std::vector<std::string> errs(n_inst);
  std::vector<char> ok(n_inst, 0);
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t n_thr = std::min<size_t>(std::min<size_t>(hw, 32), uniq.size());
  auto work = [&](size_t t) {
    for (size_t i = t; i < uniq.size(); i += n_thr) {
      const size_t j = uniq[i];
      const ci_instance& I = in[G.insts[j]];
      ok[j] = build_plan(I.mesh.num_nodes, I.mesh.num_elements, I.mesh.nodes_per_element,
                         I.mesh.xloc, I.mesh.element_nodes, G.chunk_elements, G.chunk_nodes, kDefaultTargetCtas,
                         &built[j], &errs[j]);
    }
  };
  if (n_thr <= 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (size_t t = 0; t < n_thr; t++) th.emplace_back(work, t);
    for (auto& t : th) t.join();
  }
  for (size_t u : uniq)
    if (!ok[u]) return fail(CI_ERR_INVALID, "instance " + std::to_string(G.insts[u]) + ": " + errs[u]);
  std::vector<const Plan*> plans(n_inst);
  for (size_t j = 0; j < n_inst; j++) plans[j] = &built[src[j]];
  // sizes and offsets
  G.N = G.E = G.C = 0;
  G.S = G.Lt = 0;
  G.max_local = 0;
  for (size_t j = 0; j < plans.size(); j++) {
    Inst& T = b->inst[G.insts[j]];
    const Plan& P = *plans[j];
    T.node_off = G.N;
    T.elem_off = G.E;
    T.node_orig = P.node_orig;
    T.elem_orig = P.elem_orig;
    G.N += P.N;
    G.E += P.E;
    G.C += P.n_chunks;
    G.S += P.slot_row[P.N];
    G.Lt += (long long)P.local_gid.size();
    G.max_local = std::max(G.max_local, P.max_local);
  }
  const int npe = G.npe;
  std::vector<ChunkInfo> chunks;
  std::vector<uint16_t> conn((size_t)npe * G.E);
  std::vector<uint8_t> color;
  std::vector<int> lgid, lslot, lsrow, slot_row, bnd, node_inst;
  std::vector<float> lx0(3 * (size_t)G.Lt), d0f;
  std::vector<double> d0, v0(3 * (size_t)G.N);
  std::vector<ElemParams> eps;
  std::vector<NodeParams> nps;
  std::vector<int> nsteps;
  long long s_off = 0, l_off = 0;
  slot_row.reserve(G.N + 1);
  G.max_steps = 0;
  for (size_t j = 0; j < plans.size(); j++) {
    const Plan& P = *plans[j];
    Inst& T = b->inst[G.insts[j]];
    for (ChunkInfo c : P.chunks) {
      c.elem_begin += T.elem_off;
      c.elem_end += T.elem_off;
      c.own_begin += T.node_off;
      c.local_begin += (int)l_off;
      c.slot_begin += (int)s_off;
      c.inst = (int)j;
      chunks.push_back(c);
    }
    for (int a = 0; a < npe; a++)
      std::memcpy(&conn[(size_t)a * G.E + T.elem_off], &P.conn_local[(size_t)a * P.E],
                  sizeof(uint16_t) * P.E);
    color.insert(color.end(), P.color.begin(), P.color.end());
    for (size_t l = 0; l < P.local_gid.size(); l++) {
      lgid.push_back(P.local_gid[l] + T.node_off);
      lslot.push_back(P.local_slot[l] + (int)s_off);
      lsrow.push_back(P.local_srow[2 * l] + (int)s_off);
      lsrow.push_back(P.local_srow[2 * l + 1] + (int)s_off);
    }
    for (int n = 0; n < P.N; n++) {
      slot_row.push_back(P.slot_row[n] + (int)s_off);
      if (P.slot_row[n + 1] - P.slot_row[n] > 1) bnd.push_back(n + T.node_off);
      node_inst.push_back((int)j);
      const int o = P.node_orig[n];
      const double* x = &T.X[3 * (size_t)o];
      const double d = T.wall.normal[0] * x[0] + T.wall.normal[1] * x[1] +
                       T.wall.normal[2] * x[2] - T.wall.offset;
      d0.push_back(d);
      d0f.push_back((float)d);
      for (int k = 0; k < 3; k++) v0[(size_t)k * G.N + T.node_off + n] = T.vel[k];
    }
    // chunk-relative reference coordinates
    for (int c = 0; c < P.n_chunks; c++) {
      const ChunkInfo& ch = P.chunks[c];
      const int o = P.node_orig[P.local_gid[ch.local_begin]];
      for (int l = 0; l < ch.n_local; l++) {
        const int lb = ch.local_begin + l;
        const int n = P.node_orig[P.local_gid[lb]];
        for (int k = 0; k < 3; k++)
          lx0[(size_t)k * G.Lt + l_off + lb] = (float)(T.X[3 * (size_t)n + k] - T.X[3 * (size_t)o + k]);
      }
    }
    s_off += P.slot_row[P.N];
    l_off += (long long)P.local_gid.size();
    eps.push_back(make_ep(T.mat, T.dt));
    nps.push_back(make_np(T.wall, opt.gravity, T.dt, P.N));
    nsteps.push_back(T.nsteps);
    G.max_steps = std::max(G.max_steps, T.nsteps);
  }
  slot_row.push_back((int)s_off);
  G.n_bnd = (int)bnd.size();
  G.smem = 40 * ((size_t)G.max_local + 2);
  cudaStream_t st = G.stream;
  CB_CUDA(G.chunks.upload(chunks, st));
  CB_CUDA(G.conn.upload(conn, st));
  CB_CUDA(G.color.upload(color, st));
  CB_CUDA(G.lgid.upload(lgid, st));
  CB_CUDA(G.lslot.upload(lslot, st));
  CB_CUDA(G.lsrow.upload(lsrow, st));
  CB_CUDA(G.slot_row.upload(slot_row, st));
  CB_CUDA(G.bnd.upload(bnd, st));
  CB_CUDA(G.node_inst.upload(node_inst, st));
  CB_CUDA(G.lx0.upload(lx0, st));
  CB_CUDA(G.d0.upload(d0, st));
  CB_CUDA(G.d0f.upload(d0f, st));
  CB_CUDA(G.inst_ep.upload(eps, st));
  CB_CUDA(G.inst_np.upload(nps, st));
  CB_CUDA(G.inst_nsteps.upload(nsteps, st));
  CB_CUDA(G.v0.upload(v0, st));
  CB_CUDA(G.va.alloc(3 * (size_t)G.N));
  const size_t N = G.N, E = G.E;
  CB_CUDA(G.ua.alloc(3 * N));
  CB_CUDA(G.ub.alloc(3 * N));
  CB_CUDA(G.vb.alloc(3 * N));
  CB_CUDA(G.slot0.alloc(3 * (size_t)G.S));
  CB_CUDA(G.slot1.alloc(3 * (size_t)G.S));
  CB_CUDA(G.mass.alloc(N));
  CB_CUDA(G.acc.alloc(3 * N));
  CB_CUDA(G.contact.alloc(N));
  CB_CUDA(G.sig_a.alloc(E * G.nq));
  CB_CUDA(G.sig_b.alloc(E * G.nq));
  CB_CUDA(G.epbar.alloc(E * G.nq));
  CB_CUDA(G.work.alloc(4 * (size_t)G.C));
  CB_CUDA(G.status.alloc(1));
  CB_CUDA(G.step_ctr.alloc(1));
  CB_CUDA(G.peak.alloc(G.insts.size()));
  CB_CUDA(npe == 4 ? configure<4>((int)G.smem) : configure<10>((int)G.smem));
  CB_CUDA(cudaStreamSynchronize(st));
  return CI_OK;
}

int capture_graph(Group& G) {
  if (G.graph) cudaGraphExecDestroy(G.graph);
  G.graph = nullptr;
  cudaGraph_t g = nullptr;
  CB_CUDA(cudaStreamBeginCapture(G.stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < kGraphSteps && err == cudaSuccess; i++) {
    const FusedArgs F = group_args(G, i);
    err = G.npe == 4 ? launch_batch<4>(G, F) : launch_batch<10>(G, F);
  }
  if (err == cudaSuccess) {
    k_tick<<<1, 1, 0, G.stream>>>(G.step_ctr.p, kGraphSteps);
    err = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamEndCapture(G.stream, &g);
  if (err != cudaSuccess) return fail(CI_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(err));
  if (e2 != cudaSuccess) return fail(CI_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e2));
  err = cudaGraphInstantiate(&G.graph, g, 0);
  cudaGraphDestroy(g);
  if (err != cudaSuccess) return fail(CI_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(err));
  return CI_OK;
}

// Reset to the initial state, lumped mass, a0 and half step; then (if launch) all
// steps with the plain graph.
int enqueue_run(Group& G, bool launch = true) {
  cudaStream_t st = G.stream;
  const size_t N = G.N, E = G.E;
  CB_CUDA(cudaMemsetAsync(G.ua.p, 0, sizeof(double) * 3 * N, st));
  CB_CUDA(cudaMemcpyAsync(G.va.p, G.v0.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, st));
  CB_CUDA(cudaMemsetAsync(G.sig_a.p, 0, sizeof(float4) * E * G.nq, st));
  CB_CUDA(cudaMemsetAsync(G.sig_b.p, 0, sizeof(float2) * E * G.nq, st));
  CB_CUDA(cudaMemsetAsync(G.epbar.p, 0, sizeof(float) * E * G.nq, st));
  CB_CUDA(cudaMemsetAsync(G.contact.p, 0, N, st));
  CB_CUDA(cudaMemsetAsync(G.work.p, 0, sizeof(double) * 4 * G.C, st));
  CB_CUDA(cudaMemsetAsync(G.status.p, 0, sizeof(unsigned int), st));
  CB_CUDA(cudaMemsetAsync(G.step_ctr.p, 0, sizeof(int), st));
  CB_CUDA(cudaMemsetAsync(G.peak.p, 0, sizeof(float) * G.insts.size(), st));
  DevPlan P{};
  P.chunks = G.chunks.p;
  P.conn_local = G.conn.p;
  P.color = G.color.p;
  P.local_gid = G.lgid.p;
  P.local_slot = G.lslot.p;
  P.local_srow = reinterpret_cast<const int2*>(G.lsrow.p);
  P.local_x0 = G.lx0.p;
  P.slot_row = G.slot_row.p;
  P.E = G.E;
  P.N = G.N;
  P.Lt = (int)G.Lt;
  DevState D{};
  for (int k = 0; k < 3; k++) {
    D.u[k] = G.ua.p + k * N;
    D.v[k] = G.va.p + k * N;
    D.slot_f[k] = G.slot0.p + k * (size_t)G.S;
  }
  D.status = G.status.p;
  D.chunk_work = G.work.p;
  D.inst_ep = G.inst_ep.p;
  const ElemParams p0{};
  if (G.npe == 4)
    k_elem<4, EM_MASS_HRZ, 256><<<G.C, 256, G.smem, st>>>(P, D, p0);
  else
    k_elem<10, EM_MASS_HRZ, 256><<<G.C, 256, G.smem, st>>>(P, D, p0);
  CB_CUDA(cudaGetLastError());
  k_mass_sum<<<(G.N + 255) / 256, 256, 0, st>>>(G.slot0.p, G.slot_row.p, G.mass.p, G.N);
  CB_CUDA(cudaGetLastError());
  NodeArrays A{};
  for (int k = 0; k < 3; k++) {
    A.u[k] = G.ua.p + k * N;
    A.v[k] = G.va.p + k * N;
    A.acc[k] = G.acc.p + k * N;
  }
  A.mass = G.mass.p;
  A.d0 = G.d0.p;
  A.contact = G.contact.p;
  A.status = G.status.p;
  NodeParams np0{};
  np0.N = G.N;
  k_node_init<true><<<(G.N + 255) / 256, 256, 0, st>>>(A, np0, G.inst_np.p, G.node_inst.p,
                                                       G.d0f.p);
  CB_CUDA(cudaGetLastError());
  if (launch) {
    // all global steps: max_steps + 1 (the last instance's boundary finalisation)
    const int total = G.max_steps + 1;
    for (int done = 0; done < total; done += kGraphSteps) CB_CUDA(cudaGraphLaunch(G.graph, st));
  }
  return CI_OK;
}

// enqueue_run's preparation, then graphs of `per_graph` steps covering `total` steps
int enqueue_run_graph(Group& G, int total, int per_graph) {
  const int rc = enqueue_run(G, false);
  if (rc) return rc;
  for (int done = 0; done < total; done += per_graph) CB_CUDA(cudaGraphLaunch(G.graph, G.stream));
  return CI_OK;
}

// Project autotuner: times `steps` steps of candidate tile shapes on the group's own
// instances from their initial state and keeps the fastest.  Stage 1 picks the plan --
// elements per chunk (each instance's own split, or chunks bounded by nodes only) and
// local-node budget -- at the default CTA shape; stage 2 the CTA size and lanes per
// tet10 element for that plan.  Options fixed by the caller are not varied.  The group
// is left built with the winner (graph not captured).
int trial_shape(Group& G, int graphs, cudaEvent_t e0, cudaEvent_t e1, float* ms_per_step) {
  int rc;
  if ((rc = capture_graph(G))) return rc;
  if ((rc = enqueue_run(G, false))) return rc;
  CB_CUDA(cudaGraphLaunch(G.graph, G.stream));  // warm-up: uploads the graph
  CB_CUDA(cudaEventRecord(e0, G.stream));
  for (int r = 0; r < graphs; r++) CB_CUDA(cudaGraphLaunch(G.graph, G.stream));
  CB_CUDA(cudaEventRecord(e1, G.stream));
  CB_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  CB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  unsigned int st = 0;
  CB_CUDA(cudaMemcpy(&st, G.status.p, sizeof(st), cudaMemcpyDeviceToHost));
  if (st & ST_DEGENERATE) return fail(CI_ERR_DEGENERATE, "an element has det J <= 0");
  if (st & ST_NONFINITE) return fail(CI_ERR_NONFINITE, "non-finite nodal state");
  *ms_per_step = ms / (float)(graphs * kGraphSteps);
  return CI_OK;
}

int autotune_group(ci_batch* b, Group& G, const ci_instance* in, const ci_options& opt) {
  const std::vector<int> ces = opt.chunk_elements ? std::vector<int>{opt.chunk_elements}
                                                  : std::vector<int>{0, 4096};
  const std::vector<int> cns = opt.chunk_nodes ? std::vector<int>{opt.chunk_nodes}
                                               : std::vector<int>{512, 768, 896, 1024};
  const std::vector<int> bss = opt.block_threads ? std::vector<int>{opt.block_threads}
                                                 : std::vector<int>{64, 128, 256};
  const std::vector<int> lanes = (G.npe == 4 || opt.elem_lanes) ? std::vector<int>{G.elem_lanes}
                                                                : std::vector<int>{1, 4};
  const int graphs = std::max(1, (opt.autotune_steps + kGraphSteps - 1) / kGraphSteps);
  cudaEvent_t e0, e1;
  CB_CUDA(cudaEventCreate(&e0));
  CB_CUDA(cudaEventCreate(&e1));
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } ev{e0, e1};
  int rc;
  float best = 0.f, ms = 0.f;
  int best_ce = ces[0], best_cn = cns[0];
  for (int ce : ces)
    for (int cn : cns) {
      G.chunk_elements = ce;
      G.chunk_nodes = cn;
      if ((rc = build_group(b, G, in, opt))) return rc;
      if ((rc = trial_shape(G, graphs, e0, e1, &ms))) return rc;
      if (best == 0.f || ms < best) {
        best = ms;
        best_ce = ce;
        best_cn = cn;
      }
    }
  if (G.chunk_elements != best_ce || G.chunk_nodes != best_cn) {
    G.chunk_elements = best_ce;
    G.chunk_nodes = best_cn;
    if ((rc = build_group(b, G, in, opt))) return rc;
  }
  const int bs0 = G.block_threads, ln0 = G.elem_lanes;
  int best_bs = bs0, best_ln = ln0;
  for (int bs : bss)
    for (int ln : lanes) {
      if (bs == bs0 && ln == ln0) continue;  // measured in stage 1
      G.block_threads = bs;
      G.elem_lanes = ln;
      if ((rc = trial_shape(G, graphs, e0, e1, &ms))) return rc;
      if (ms < best) {
        best = ms;
        best_bs = bs;
        best_ln = ln;
      }
    }
  G.block_threads = best_bs;
  G.elem_lanes = best_ln;
  G.tuned_ms_per_step = best;
  return CI_OK;
}

// Displacement of every node after k = *step_ctr global steps, FP32, into
// snap[(k / every - 1)][node][3] (plan order).  A node of an instance still stepping
// is completed from S^{k-1} and the halo of step k-1 exactly as step k will do it;
// instances that have finished (k > nsteps) hold their final state in buffer nsteps & 1.
// Displacement of node n at the snapshot the current tick ends (the state after
// k = *step_ctr steps of its instance, or its final state once it has stopped); false
// outside the snapshot range.
__device__ __forceinline__ bool snapshot_u(const FusedArgs& A0, const FusedArgs& A1,
                                           const int* node_inst, int n, int every, int max_snaps,
                                           double (&u)[3], int& si, int& inst) {
  const int k = *A0.step_ctr;
  si = k / every - 1;
  if (si < 0 || si >= max_snaps) return false;
  inst = node_inst[n];
  const int ns = A0.inst_nsteps[inst];
  // A0: views with cur = buffer A (even k), A1: cur = buffer B
  if (k > ns) {
    const FusedArgs& F = (ns & 1) ? A1 : A0;
    for (int c = 0; c < 3; c++) u[c] = F.u_cur[c][n];
  } else {
    // the step-k view: prv holds S^{k-1}, halo_prv the halo of step k-1
    const FusedArgs& F = (k & 1) ? A1 : A0;
    double v[3];
    float a[3], uf[3], vf[3];
    bool hit;
    complete_node(F, F.inst_np[inst], n, F.P.slot_row[n], F.P.slot_row[n + 1], u, v, a, hit, uf,
                  vf);
  }
  return true;
}

__global__ void k_snapshot(FusedArgs A0, FusedArgs A1, const int* node_inst, int N, int every,
                           float* snap, int max_snaps) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double u[3];
  int si, inst;
  if (!snapshot_u(A0, A1, node_inst, n, every, max_snaps, u, si, inst)) return;
  float* o = snap + ((size_t)si * N + n) * 3;
  o[0] = (float)u[0];
  o[1] = (float)u[1];
  o[2] = (float)u[2];
}

// Running maximum per instance of the nodal displacement norm at the snapshot times,
// from the FP32 displacement the snapshots hold; non-negative floats order like their
// bit patterns, so the integer maximum is exact and independent of the order.
__global__ void k_snapshot_peak(FusedArgs A0, FusedArgs A1, const int* node_inst, int N, int every,
                                int max_snaps, float* inst_peak) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double u[3];
  int si, inst;
  if (!snapshot_u(A0, A1, node_inst, n, every, max_snaps, u, si, inst)) return;
  const float x = (float)u[0], y = (float)u[1], z = (float)u[2];
  const float m = sqrtf(x * x + y * y + z * z);
  atomicMax(reinterpret_cast<int*>(inst_peak) + inst, __float_as_int(m));
}

// Largest equivalent plastic strain per instance (one CTA per chunk, integer maximum of
// the non-negative float bits).
__global__ void k_peak_epbar(const ChunkInfo* chunks, const float* epbar, int nq, float* inst_peak) {
  const ChunkInfo ch = chunks[blockIdx.x];
  float m = 0.f;
  for (long long i = (long long)ch.elem_begin * nq + threadIdx.x; i < (long long)ch.elem_end * nq;
       i += blockDim.x)
    m = fmaxf(m, epbar[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(inst_peak) + ch.inst, __float_as_int(m));
}

}  // namespace

extern "C" {

int ci_batch_create(const ci_instance* inst, int n, const ci_options* opt_in, ci_batch** out) {
  if (!inst || n <= 0 || !out) return fail(CI_ERR_INVALID, "ci_batch_create: no instances");
  *out = nullptr;
  ci_options opt;
  if (opt_in)
    opt = *opt_in;
  else
    ci_default_options(&opt);
  std::unique_ptr<ci_batch> b(new ci_batch());
  b->device = opt.device;
  CB_CUDA(cudaSetDevice(b->device));
  b->inst.resize(n);
  for (int i = 0; i < n; i++) {
    const ci_instance& I = inst[i];
    const int npe = I.mesh.nodes_per_element;
    if (npe != 4 && npe != 10) return fail(CI_ERR_UNSUPPORTED, "instance with npe not 4 or 10");
    if (!(I.dt > 0.0) || !(I.t_end >= 0.0)) return fail(CI_ERR_INVALID, "instance dt/t_end");
    if (I.mat.beta != 0.0) return fail(CI_ERR_UNSUPPORTED, "only isotropic hardening (beta = 0)");
    Inst& T = b->inst[i];
    T.group = npe == 4 ? 0 : 1;
    T.N = I.mesh.num_nodes;
    T.E = I.mesh.num_elements;
    T.npe = npe;
    T.dt = I.dt;
    long long ns = 0;
    for (double t = 0.0; t <= I.t_end; t += I.dt) ns++;  // the reference's loop count
    if (ns > (1 << 30)) return fail(CI_ERR_TOO_LARGE, "instance needs too many steps");
    T.nsteps = (int)ns;
    T.X.resize(3 * (size_t)T.N);
    for (int k = 0; k < 3 * T.N; k++) T.X[k] = I.mesh.xloc[k] + I.pos[k % 3];
    T.mat = I.mat;
    T.wall = I.wall;
    for (int k = 0; k < 3; k++) T.vel[k] = I.vel[k];
  }
  for (int gi = 0; gi < 2; gi++) {
    std::unique_ptr<Group> G(new Group());
    G->npe = gi == 0 ? 4 : 10;
    G->nq = gi == 0 ? 1 : 4;
    for (int i = 0; i < n; i++)
      if (b->inst[i].group == gi) {
        b->inst[i].index = (int)G->insts.size();
        G->insts.push_back(i);
      }
    if (G->insts.empty()) continue;
    G->block_threads = opt.block_threads ? opt.block_threads : 128;
    G->elem_lanes = opt.elem_lanes ? opt.elem_lanes : 4;
    G->chunk_nodes = opt.chunk_nodes ? opt.chunk_nodes : 896;
    G->chunk_elements = opt.chunk_elements;
    if (G->block_threads != 64 && G->block_threads != 128 && G->block_threads != 256)
      return fail(CI_ERR_INVALID, "block_threads must be 64, 128 or 256");
    if (G->elem_lanes != 1 && G->elem_lanes != 4)
      return fail(CI_ERR_INVALID, "elem_lanes must be 1 or 4");
    CB_CUDA(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    int rc = opt.autotune_steps > 0 ? autotune_group(b.get(), *G, inst, opt)
                                    : build_group(b.get(), *G, inst, opt);
    if (rc) return rc;
    if ((rc = capture_graph(*G))) return rc;
    b->g[gi] = std::move(G);
  }
  CB_CUDA(cudaEventCreate(&b->ev0));
  CB_CUDA(cudaEventCreate(&b->ev1));
  *out = b.release();
  return CI_OK;
}

int ci_batch_run(ci_batch* b, float* device_ms) {
  if (!b) return fail(CI_ERR_INVALID, "null batch");
  CB_CUDA(cudaSetDevice(b->device));
  // both groups start after ev0 and end before ev1 (device time of the whole batch)
  cudaStream_t s0 = b->g[0] ? b->g[0]->stream : b->g[1]->stream;
  CB_CUDA(cudaEventRecord(b->ev0, s0));
  for (int gi = 0; gi < 2; gi++)
    if (b->g[gi]) {
      CB_CUDA(cudaStreamWaitEvent(b->g[gi]->stream, b->ev0, 0));
      const int rc = enqueue_run(*b->g[gi]);
      if (rc) return rc;
    }
  std::vector<cudaEvent_t> ends;
  for (int gi = 0; gi < 2; gi++)
    if (b->g[gi] && b->g[gi]->stream != s0) {
      cudaEvent_t e;
      CB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      CB_CUDA(cudaEventRecord(e, b->g[gi]->stream));
      CB_CUDA(cudaStreamWaitEvent(s0, e, 0));
      ends.push_back(e);
    }
  CB_CUDA(cudaEventRecord(b->ev1, s0));
  CB_CUDA(cudaEventSynchronize(b->ev1));
  for (cudaEvent_t e : ends) cudaEventDestroy(e);
  CB_CUDA(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
  if (device_ms) *device_ms = b->last_ms;
  for (int gi = 0; gi < 2; gi++)
    if (b->g[gi]) {
      unsigned int st = 0;
      CB_CUDA(cudaMemcpy(&st, b->g[gi]->status.p, sizeof(st), cudaMemcpyDeviceToHost));
      if (st & ST_DEGENERATE) return fail(CI_ERR_DEGENERATE, "an element has det J <= 0");
      if (st & ST_NONFINITE) return fail(CI_ERR_NONFINITE, "non-finite nodal state");
    }
  b->done = true;
  return CI_OK;
}

int ci_batch_tuning(ci_batch* b, int npe, int* chunk_elements, int* chunk_nodes, int* block_threads,
                    int* elem_lanes, float* trial_ms_per_step) {
  if (!b || (npe != 4 && npe != 10)) return fail(CI_ERR_INVALID, "ci_batch_tuning: bad arguments");
  const Group* G = b->g[npe == 4 ? 0 : 1].get();
  if (!G) return fail(CI_ERR_INVALID, "ci_batch_tuning: the batch has no instance of that type");
  if (chunk_elements) *chunk_elements = G->chunk_elements;
  if (chunk_nodes) *chunk_nodes = G->chunk_nodes;
  if (block_threads) *block_threads = G->block_threads;
  if (elem_lanes) *elem_lanes = G->npe == 10 ? G->elem_lanes : 1;
  if (trial_ms_per_step) *trial_ms_per_step = G->tuned_ms_per_step;
  return CI_OK;
}

int ci_batch_get_state(ci_batch* b, int i, double* x, double* v, float* epbar,
                       unsigned char* contact, long long* nsteps) {
  if (!b || i < 0 || i >= (int)b->inst.size()) return fail(CI_ERR_INVALID, "bad instance index");
  if (!b->done) return fail(CI_ERR_INVALID, "ci_batch_run has not completed");
  CB_CUDA(cudaSetDevice(b->device));
  const Inst& T = b->inst[i];
  const Group& G = *b->g[T.group];
  const int N = T.N, E = T.E, nq = G.nq;
  // final state in buffer A for an even step count, B for an odd one
  const bool a = (T.nsteps & 1) == 0;
  std::vector<double> hu(3 * (size_t)N), hv(3 * (size_t)N);
  for (int k = 0; k < 3; k++) {
    CB_CUDA(cudaMemcpy(&hu[(size_t)k * N], (a ? G.ua.p : G.ub.p) + (size_t)k * G.N + T.node_off,
                       sizeof(double) * N, cudaMemcpyDeviceToHost));
    CB_CUDA(cudaMemcpy(&hv[(size_t)k * N], (a ? G.va.p : G.vb.p) + (size_t)k * G.N + T.node_off,
                       sizeof(double) * N, cudaMemcpyDeviceToHost));
  }
  std::vector<unsigned char> hc(N);
  CB_CUDA(cudaMemcpy(hc.data(), G.contact.p + T.node_off, N, cudaMemcpyDeviceToHost));
  std::vector<float> hep((size_t)E * nq);
  CB_CUDA(cudaMemcpy(hep.data(), G.epbar.p + (size_t)T.elem_off * nq, sizeof(float) * hep.size(),
                     cudaMemcpyDeviceToHost));
  for (int p = 0; p < N; p++) {
    const int o = T.node_orig[p];
    for (int k = 0; k < 3; k++) {
      if (x) x[3 * (size_t)o + k] = T.X[3 * (size_t)o + k] + hu[(size_t)k * N + p];
      if (v) v[3 * (size_t)o + k] = hv[(size_t)k * N + p];
    }
    if (contact) contact[o] = hc[p];
  }
  if (epbar)
    for (int pe = 0; pe < E; pe++)
      for (int q = 0; q < nq; q++)
        epbar[(size_t)T.elem_orig[pe] * nq + q] = hep[(size_t)pe * nq + q];
  if (nsteps) *nsteps = T.nsteps;
  return CI_OK;
}

}  // extern "C"

namespace {

// Runs every instance in graphs of `every` steps, each followed by the step tick and
// tail(G) (kernels on G.stream, captured into the graph); the device time goes to
// *device_ms.  One element type per batch.
template <class Tail>
int run_intervals(ci_batch* b, int every, float* device_ms, const char* what, Tail tail) {
  if (b->g[0] && b->g[1])
    return fail(CI_ERR_UNSUPPORTED, std::string(what) + ": one element type per batch");
  CB_CUDA(cudaSetDevice(b->device));
  Group& G = *(b->g[0] ? b->g[0] : b->g[1]);
  if (G.graph) cudaGraphExecDestroy(G.graph);
  G.graph = nullptr;
  cudaGraph_t g = nullptr;
  CB_CUDA(cudaStreamBeginCapture(G.stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < every && err == cudaSuccess; i++) {
    const FusedArgs F = group_args(G, i);
    err = G.npe == 4 ? launch_batch<4>(G, F) : launch_batch<10>(G, F);
  }
  if (err == cudaSuccess) {
    k_tick<<<1, 1, 0, G.stream>>>(G.step_ctr.p, every);
    tail(G);
    err = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamEndCapture(G.stream, &g);
  if (err != cudaSuccess || e2 != cudaSuccess)
    return fail(CI_ERR_CUDA, std::string(what) + " capture: " +
                                 cudaGetErrorString(err != cudaSuccess ? err : e2));
  err = cudaGraphInstantiate(&G.graph, g, 0);
  cudaGraphDestroy(g);
  if (err != cudaSuccess) return fail(CI_ERR_CUDA, std::string(what) + " graph: " + cudaGetErrorString(err));
  CB_CUDA(cudaEventRecord(b->ev0, G.stream));
  // ceil((max_steps + 1) / every) graphs of `every` steps, prepared like a normal run
  {
    const int rc = enqueue_run_graph(G, G.max_steps + 1, every);
    if (rc) return rc;
  }
  CB_CUDA(cudaEventRecord(b->ev1, G.stream));
  CB_CUDA(cudaEventSynchronize(b->ev1));
  CB_CUDA(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
  if (device_ms) *device_ms = b->last_ms;
  // restore the plain graph for later ci_batch_run calls
  const int rc = capture_graph(G);
  if (rc) return rc;
  unsigned int stw = 0;
  CB_CUDA(cudaMemcpy(&stw, G.status.p, sizeof(stw), cudaMemcpyDeviceToHost));
  if (stw & ST_NONFINITE) return fail(CI_ERR_NONFINITE, "non-finite nodal state");
  b->done = true;
  return CI_OK;
}

}  // namespace

extern "C" {

int ci_batch_run_snapshots(ci_batch* b, int every, float* d_snap, int max_snaps, float* device_ms) {
  if (!b || every <= 0 || (every & 1) || !d_snap || max_snaps <= 0)
    return fail(CI_ERR_INVALID, "ci_batch_run_snapshots: needs an even interval and a buffer");
  return run_intervals(b, every, device_ms, "ci_batch_run_snapshots", [&](Group& G) {
    k_snapshot<<<(G.N + 255) / 256, 256, 0, G.stream>>>(group_args(G, 0), group_args(G, 1),
                                                        G.node_inst.p, G.N, every, d_snap, max_snaps);
  });
}

int ci_batch_run_peaks(ci_batch* b, int every, int max_snaps, float* peak_disp, float* peak_epbar,
                       float* device_ms) {
  if (!b || every <= 0 || (every & 1) || max_snaps <= 0)
    return fail(CI_ERR_INVALID, "ci_batch_run_peaks: needs an even interval");
  int rc = run_intervals(b, every, device_ms, "ci_batch_run_peaks", [&](Group& G) {
    k_snapshot_peak<<<(G.N + 255) / 256, 256, 0, G.stream>>>(group_args(G, 0), group_args(G, 1),
                                                             G.node_inst.p, G.N, every, max_snaps,
                                                             G.peak.p);
  });
  if (rc) return rc;
  Group& G = *(b->g[0] ? b->g[0] : b->g[1]);
  const size_t ni = G.insts.size();
  DBuf<float> d_ep;
  CB_CUDA(d_ep.alloc(ni));
  CB_CUDA(cudaMemsetAsync(d_ep.p, 0, sizeof(float) * ni, G.stream));
  k_peak_epbar<<<G.C, 256, 0, G.stream>>>(G.chunks.p, G.epbar.p, G.nq, d_ep.p);
  CB_CUDA(cudaGetLastError());
  std::vector<float> hd(ni), he(ni);
  CB_CUDA(cudaMemcpyAsync(hd.data(), G.peak.p, sizeof(float) * ni, cudaMemcpyDeviceToHost, G.stream));
  CB_CUDA(cudaMemcpyAsync(he.data(), d_ep.p, sizeof(float) * ni, cudaMemcpyDeviceToHost, G.stream));
  CB_CUDA(cudaStreamSynchronize(G.stream));
  for (size_t k = 0; k < ni; k++) {
    if (peak_disp) peak_disp[G.insts[k]] = hd[k];
    if (peak_epbar) peak_epbar[G.insts[k]] = he[k];
  }
  return CI_OK;
}

/* Plan order of instance i's nodes: perm[p] = caller node of plan node p. */
int ci_batch_node_order(ci_batch* b, int i, int* perm, int* node_offset) {
  if (!b || i < 0 || i >= (int)b->inst.size() || !perm) return fail(CI_ERR_INVALID, "bad argument");
  const Inst& T = b->inst[i];
  std::memcpy(perm, T.node_orig.data(), sizeof(int) * T.N);
  if (node_offset) *node_offset = T.node_off;
  return CI_OK;
}

int ci_batch_destroy(ci_batch* b) {
  if (!b) return CI_OK;
  cudaSetDevice(b->device);
  for (int gi = 0; gi < 2; gi++)
    if (b->g[gi]) cudaStreamSynchronize(b->g[gi]->stream);
  delete b;
  return CI_OK;
}

}  // extern "C"
