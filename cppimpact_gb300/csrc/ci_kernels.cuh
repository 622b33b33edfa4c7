// ci_kernels.cuh -- sm_103a kernels of the explicit impact step.
//
// Fused step (one launch per step, captured in CUDA graphs; one CTA per chunk, see
// ci_plan.h).  Each CTA (1) completes S^n of every local node of its chunk from S^{n-1}
// and the previous step's halo (slots summed in fixed order; a = -f/m, planar penalty
// wall and gravity, include/dynamics_kernels.h:150-168, include/wall.h:37-43; FP64
// central-difference update, include/dynamics.h:477-503) and stages it in shared
// memory, (2) computes the element internal force matrix-free in FP32
// (FEAnalysis::calculate_f_internal, include/analysis.h:321-382, without forming B or
// K_e) with the J2 update, accumulating node forces in shared memory colour by colour,
// (3) writes one partial sum per (chunk, local node) slot:
//   k_step_qp10 : tet10, 4 lanes per element (one per Gauss point), reduce-scatter
//   k_step_t10  : tet10, one thread per element, barycentric form
//   k_step      : tet4, one thread per element
//   k_finalize_nodes : S^N after the last step of a call
// Two-kernel path and one-shot entry points: k_elem (element work to slots) + k_node
// (one thread per node); k_elem<MASS_*> + k_mass_sum: lumped mass, once
// (include/analysis.h:136-162).
//
// No float atomics anywhere: every floating-point sum has a fixed order.
#pragma once
#include <cstdint>

#include "ci_fpconv.h"
#include "ci_plan.h"

namespace ci {


enum ElemMode { EM_J2 = 0, EM_REFCOMPAT = 1, EM_MASS_ROWSUM = 2, EM_MASS_HRZ = 3 };

enum StatusBits { ST_DEGENERATE = 1u, ST_NONFINITE = 2u, ST_FLOW_TIMEOUT = 8u };

struct DevPlan {
  const ChunkInfo* chunks;
  const uint16_t* conn_local;  // [npe][E]
  const uint8_t* color;        // [E]
  const int* local_gid;        // [Lt]
  const int* local_slot;       // [Lt]
  const float* local_x0;       // [3][Lt] reference coordinates relative to the chunk origin
  const int* slot_row;         // [N+1]
  const int2* local_srow;      // [Lt] slot range of each local node's node
  int E, N, Lt;
};

struct ElemParams {
  float dt;
  float lambda, mu;       // Lame constants
  float sy0, H;           // yield stress, hardening modulus
  float rho;
  int accum_energy;       // accumulate work terms into chunk_work
};

struct DevState {
  double* u[3];        // displacement from the reference positions, SoA [N]
  double* v[3];        // half-step velocity, SoA [N]
  float* slot_f[3];    // partial node forces per slot, SoA [S]
  float4* sig_a;       // [E][nq] stress xx yy zz xy
  float2* sig_b;       // [E][nq] stress yz xz
  float* epbar;        // [E][nq] equivalent plastic strain
  double* chunk_work;  // [C][4] internal work, plastic work, volume, unused (running sums)
  unsigned int* status;
  const ElemParams* inst_ep;  // per-instance parameters of a batched solve (else null)
};


struct NodeParams {
  double dt;
  double g[3];
  double wall_n[3];
  double wall_k;
  float gf[3];  // g and wall normal rounded to FP32
  float nf[3];
  int N;
};

struct NodeArrays {
  double* u[3];
  double* v[3];
  const float* slot_f[3];
  const int* slot_row;
  const float* mass;
  const double* d0;        // wall_n . X - wall_offset per node
  unsigned char* contact;  // bit0 current, bit1 ever
  float* acc[3];           // last acceleration (written when STORE_ACC)
  unsigned int* status;
};

// ---------------------------------------------------------------------------
// Element geometry: the reference parametrisation (include/tetrahedral.h:182-250,
// 521-549): barycentrics L = (xi, eta, 1-xi-eta-zeta, zeta) for corners 0..3 and the
// CalculiX edge order 4:(0,1) 5:(1,2) 6:(2,0) 7:(0,3) 8:(1,3) 9:(2,3).
// ---------------------------------------------------------------------------
template <int NPE>
struct Rule;

template <>
struct Rule<4> {
  static constexpr int NQ = 1;
  static constexpr float W = 1.0f / 6.0f;
  __device__ __forceinline__ static void grad(int, float G[4][3]) {
    G[0][0] = -1.f; G[0][1] = -1.f; G[0][2] = -1.f;
    G[1][0] = 1.f;  G[1][1] = 0.f;  G[1][2] = 0.f;
    G[2][0] = 0.f;  G[2][1] = 1.f;  G[2][2] = 0.f;
    G[3][0] = 0.f;  G[3][1] = 0.f;  G[3][2] = 1.f;
  }
  __device__ __forceinline__ static void shape(int, float N[4]) {
    N[0] = N[1] = N[2] = N[3] = 0.25f;
  }
};

template <>
struct Rule<10> {
  // 4-point Gauss rule, degree 2: a = (5 + 3 sqrt5)/20, b = (5 - sqrt5)/20, w = 1/24.
  static constexpr int NQ = 4;
  static constexpr float W = 1.0f / 24.0f;
  __device__ __forceinline__ static void bary(int q, float L[4]) {
    const float a = 0.58541019662496845f, b = 0.13819660112501052f;
    // QP q has parametric point (b,b,b), (a,b,b), (b,a,b), (b,b,a)
    const float xi = q == 1 ? a : b, eta = q == 2 ? a : b, zeta = q == 3 ? a : b;
    L[0] = xi;
    L[1] = eta;
    L[2] = q == 0 ? a : b;  // 1 - xi - eta - zeta
    L[3] = zeta;
  }
  __device__ __forceinline__ static void grad(int q, float G[10][3]) {
    float L[4];
    bary(q, L);
    const float dL[4][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {-1.f, -1.f, -1.f}, {0.f, 0.f, 1.f}};
    const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
#pragma unroll
    for (int c = 0; c < 4; c++)
#pragma unroll
      for (int j = 0; j < 3; j++) G[c][j] = (4.f * L[c] - 1.f) * dL[c][j];
#pragma unroll
    for (int k = 0; k < 6; k++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        G[4 + k][j] = 4.f * (L[ea[k]] * dL[eb[k]][j] + L[eb[k]] * dL[ea[k]][j]);
  }
  __device__ __forceinline__ static void shape(int q, float N[10]) {
    float L[4];
    bary(q, L);
    const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
#pragma unroll
    for (int c = 0; c < 4; c++) N[c] = L[c] * (2.f * L[c] - 1.f);
#pragma unroll
    for (int k = 0; k < 6; k++) N[4 + k] = 4.f * L[ea[k]] * L[eb[k]];
  }
};

// Cofactor inverse of a 3x3 (row-major), returns det (cf. inv3x3, include/physics.h:38-58).
__device__ __forceinline__ float inv3f(const float* A, float* Ai) {
  const float c00 = A[4] * A[8] - A[5] * A[7];
  const float c01 = A[5] * A[6] - A[3] * A[8];
  const float c02 = A[3] * A[7] - A[4] * A[6];
  const float det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  const float r = __frcp_rn(det);
  Ai[0] = c00 * r;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) * r;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * r;
  Ai[3] = c01 * r;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * r;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) * r;
  Ai[6] = c02 * r;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) * r;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * r;
  return det;
}

// J2 radial return with linear isotropic hardening (Simo & Hughes 1998, Box 3.1):
// trial = s + lambda tr(de) I + 2 mu de (engineering shear in de[3..5]); if the
// deviatoric norm exceeds sqrt(2/3)(sy0 + H epbar), return along the deviator.
__device__ __forceinline__ void j2_return(const ElemParams& p, float s[6], float& epbar) {
  const float pm = (s[0] + s[1] + s[2]) * (1.0f / 3.0f);
  const float d0 = s[0] - pm, d1 = s[1] - pm, d2 = s[2] - pm;
  const float nrm2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.f * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
  const float nrm = sqrtf(nrm2);
  const float f = nrm - 0.81649658092772603f * (p.sy0 + p.H * epbar);
  if (f > 0.f) {
    const float dg = f / (2.f * p.mu + (2.f / 3.f) * p.H);
    const float sc = 1.f - 2.f * p.mu * dg / nrm;
    s[0] = d0 * sc + pm;
    s[1] = d1 * sc + pm;
    s[2] = d2 * sc + pm;
    s[3] *= sc;
    s[4] *= sc;
    s[5] *= sc;
    epbar += 0.81649658092772603f * dg;
  }
}

// Element internal force (and J2 update) for element e at plan position e.
// x: current coordinates relative to the chunk origin, du: increment.
template <int NPE, int MODE>
__device__ __forceinline__ void element_force(const ElemParams& p, const DevState& S, int e, int E,
                                              const float (&x)[NPE][3], const float (&du)[NPE][3],
                                              float (&f)[NPE][3], float& wint, float& wp,
                                              float& vol) {
  using R = Rule<NPE>;
#pragma unroll
  for (int i = 0; i < NPE; i++) f[i][0] = f[i][1] = f[i][2] = 0.f;
  float ve = 0.f;  // this element's volume (vol accumulates over the thread's elements)
#pragma unroll
  for (int q = 0; q < R::NQ; q++) {
    float G[NPE][3];
    R::grad(q, G);
    float J[9];
#pragma unroll
    for (int k = 0; k < 9; k++) J[k] = 0.f;
#pragma unroll
    for (int i = 0; i < NPE; i++)
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++) J[3 * a + j] = fmaf(x[i][a], G[i][j], J[3 * a + j]);
    float Ji[9];
    const float detJ = inv3f(J, Ji);
    if (!(detJ > 0.f)) atomicOr(S.status, (unsigned)ST_DEGENERATE);
    const float wd = R::W * detJ;
    vol += wd;
    ve += wd;
    if (MODE == EM_MASS_ROWSUM || MODE == EM_MASS_HRZ) {
      float N[NPE];
      R::shape(q, N);
#pragma unroll
      for (int i = 0; i < NPE; i++) f[i][0] = fmaf(p.rho * wd, N[i], f[i][0]);
      continue;
    }
    // grad du = (sum_i du_i (x) dN_i/dxi) J^-1
    float Gu[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Gu[k] = 0.f;
#pragma unroll
    for (int i = 0; i < NPE; i++)
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++) Gu[3 * a + j] = fmaf(du[i][a], G[i][j], Gu[3 * a + j]);
    float L[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++)
        L[3 * a + b] = Gu[3 * a + 0] * Ji[0 * 3 + b] + Gu[3 * a + 1] * Ji[1 * 3 + b] +
                       Gu[3 * a + 2] * Ji[2 * 3 + b];
    const float de[6] = {L[0], L[4], L[8], L[1] + L[3], L[5] + L[7], L[2] + L[6]};
    const float tr = de[0] + de[1] + de[2];
    float s[6];
    if (MODE == EM_REFCOMPAT) {
      s[0] = p.lambda * tr + 2.f * p.mu * de[0];
      s[1] = p.lambda * tr + 2.f * p.mu * de[1];
      s[2] = p.lambda * tr + 2.f * p.mu * de[2];
      s[3] = p.mu * de[3];
      s[4] = p.mu * de[4];
      s[5] = p.mu * de[5];
      if (p.accum_energy) {
        float w = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) w = fmaf(s[k], de[k], w);
        wint = fmaf(0.5f * wd, w, wint);
      }
    } else {
      const size_t qi = (size_t)e * R::NQ + q;
      const float4 sa = S.sig_a[qi];
      const float2 sb = S.sig_b[qi];
      float ep = S.epbar[qi];
      const float s0[6] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y};
      s[0] = s0[0] + p.lambda * tr + 2.f * p.mu * de[0];
      s[1] = s0[1] + p.lambda * tr + 2.f * p.mu * de[1];
      s[2] = s0[2] + p.lambda * tr + 2.f * p.mu * de[2];
      s[3] = s0[3] + p.mu * de[3];
      s[4] = s0[4] + p.mu * de[4];
      s[5] = s0[5] + p.mu * de[5];
      const float ep0 = ep;
      j2_return(p, s, ep);
      S.sig_a[qi] = make_float4(s[0], s[1], s[2], s[3]);
      S.sig_b[qi] = make_float2(s[4], s[5]);
      S.epbar[qi] = ep;
      if (p.accum_energy) {
        float w = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) w = fmaf(s0[k] + s[k], de[k], w);
        wint = fmaf(0.5f * wd, w, wint);
        wp = fmaf(wd * (p.sy0 + p.H * ep), ep - ep0, wp);
      }
    }
    // f_i += wd sigma . dN_i/dx = sum_j P[a][j] dN_i/dxi_j with P = wd sigma J^-T
    const float Sg[9] = {s[0], s[3], s[5], s[3], s[1], s[4], s[5], s[4], s[2]};
    float Pm[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        Pm[3 * a + j] = wd * (Sg[3 * a + 0] * Ji[3 * j + 0] + Sg[3 * a + 1] * Ji[3 * j + 1] +
                              Sg[3 * a + 2] * Ji[3 * j + 2]);
#pragma unroll
    for (int i = 0; i < NPE; i++)
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++) f[i][a] = fmaf(Pm[3 * a + j], G[i][j], f[i][a]);
  }
  if (MODE == EM_MASS_HRZ && NPE == 10) {
    // HRZ for the straight-sided tet10: rho V/36 at corners, 4 rho V/27 at edges.
    const float mv = p.rho * ve;
#pragma unroll
    for (int i = 0; i < NPE; i++) f[i][0] = i < 4 ? mv * (1.f / 36.f) : mv * (4.f / 27.f);
  }
}

template <int BS>
__device__ __forceinline__ float block_sum(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x == 0)
    for (int k = 0; k < BS / 32; k++) t += red[k];
  return t;  // valid on thread 0
}

// K1 / K3.  Shared memory: x[3][Lmax] du[3][Lmax] acc[3][Lmax] floats + reduction.
template <int NPE, int MODE, int BS>
__global__ void __launch_bounds__(BS) k_elem(DevPlan P, DevState S, ElemParams p_arg) {
  extern __shared__ float sm[];
  const ChunkInfo ch = P.chunks[blockIdx.x];
  const ElemParams p = S.inst_ep ? S.inst_ep[ch.inst] : p_arg;
  const int L = ch.n_local;
  float* sx = sm;
  float* sd = sm + 3 * L;
  float* sa = sm + 6 * L;
  __shared__ float red[BS / 32];
  constexpr bool kMass = MODE == EM_MASS_ROWSUM || MODE == EM_MASS_HRZ;

  for (int l = threadIdx.x; l < L; l += BS) {
    const int lb = ch.local_begin + l;
    const int g = P.local_gid[lb];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      sx[k * L + l] = P.local_x0[(size_t)k * P.Lt + lb] + (float)S.u[k][g];
      sd[k * L + l] = kMass ? 0.f : p.dt * (float)S.v[k][g];
      sa[k * L + l] = 0.f;
    }
  }
  __syncthreads();

  float wint = 0.f, wp = 0.f, vol = 0.f;
  const int E = P.E;
  for (int w = ch.elem_begin; w < ch.elem_end; w += BS) {
    const int e = w + threadIdx.x;
    const bool act = e < ch.elem_end;
    int col = -1;
    int ln[NPE];
    float f[NPE][3];
    if (act) {
      col = P.color[e];
      float x[NPE][3], du[NPE][3];
#pragma unroll
      for (int a = 0; a < NPE; a++) {
        ln[a] = P.conn_local[(size_t)a * E + e];
#pragma unroll
        for (int k = 0; k < 3; k++) {
          x[a][k] = sx[k * L + ln[a]];
          du[a][k] = sd[k * L + ln[a]];
        }
      }
      element_force<NPE, MODE>(p, S, e, E, x, du, f, wint, wp, vol);
    }
    const int c0 = P.color[w];
    const int c1 = P.color[min(w + BS, ch.elem_end) - 1];
    for (int k = c0; k <= c1; k++) {
      __syncthreads();
      if (col == k) {
#pragma unroll
        for (int a = 0; a < NPE; a++) {
          sa[ln[a]] += f[a][0];
          if (!kMass) {
            sa[L + ln[a]] += f[a][1];
            sa[2 * L + ln[a]] += f[a][2];
          }
        }
      }
    }
  }
  __syncthreads();
  for (int l = threadIdx.x; l < L; l += BS) {
    const int s = P.local_slot[ch.local_begin + l];
    S.slot_f[0][s] = sa[l];
    if (!kMass) {
      S.slot_f[1][s] = sa[L + l];
      S.slot_f[2][s] = sa[2 * L + l];
    }
  }
  if (p.accum_energy) {
    const float t0 = block_sum<BS>(wint, red);
    const float t1 = block_sum<BS>(wp, red);
    const float t2 = block_sum<BS>(vol, red);
    if (threadIdx.x == 0) {
      double* cw = S.chunk_work + 4 * (size_t)blockIdx.x;
      cw[0] += (double)t0;
      cw[1] += (double)t1;
      cw[2] += (double)t2;
    }
  }
}

// K2: node update.  INIT: a0 from zero internal force and v += dt/2 a0
// (include/dynamics.h:454-463); otherwise one full central-difference step.
template <bool INIT, bool STORE_ACC>
__global__ void __launch_bounds__(256) k_node(NodeArrays A, NodeParams p) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= p.N) return;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  if (!INIT) {
    const int s1 = A.slot_row[n + 1];
    for (int s = A.slot_row[n]; s < s1; s++) {
      fx += A.slot_f[0][s];
      fy += A.slot_f[1][s];
      fz += A.slot_f[2][s];
    }
  }
  const float m = A.mass[n];
  const float rm = 1.0f / m;
  double a[3] = {(double)(-fx * rm) + p.g[0], (double)(-fy * rm) + p.g[1],
                 (double)(-fz * rm) + p.g[2]};
  double u[3], v[3], un[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    u[k] = A.u[k][n];
    v[k] = A.v[k][n];
    un[k] = INIT ? u[k] : fma(p.dt, v[k], u[k]);  // u + du, du = dt v
  }
  // wall at the end-of-step position (Wall::detect_contact on x + du)
  const double d = A.d0[n] + p.wall_n[0] * un[0] + p.wall_n[1] * un[1] + p.wall_n[2] * un[2];
  const unsigned char old = A.contact[n];
  unsigned char flag = old & 2;
  if (d < 0.0) {
    const double c = -d * p.wall_k / (double)m;
#pragma unroll
    for (int k = 0; k < 3; k++) a[k] = fma(c, p.wall_n[k], a[k]);
    flag = 3;
  }
  if (flag != old) A.contact[n] = flag;
  const double h = INIT ? 0.5 * p.dt : p.dt;
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double vn = fma(h, a[k], v[k]);
    finite = finite && isfinite(vn);
    A.v[k][n] = vn;
    if (!INIT) A.u[k][n] = un[k];
    if (STORE_ACC) A.acc[k][n] = (float)a[k];
  }
  if (!finite) atomicOr(A.status, (unsigned)ST_NONFINITE);
}

// ---------------------------------------------------------------------------
// Fused step (one launch per time step, no grid-wide barrier).
//
// Node state S^n = (u^n, v^{n+1/2}) is double-buffered: step n reads S^{n-1} from one
// buffer and its owner writes S^n to the other.  Every chunk writes its partial force
// on each of its local nodes to that node's slot in the halo buffer of step n.  At the
// start of step n+1 every chunk touching a node sums the node's slots in fixed chunk
// order and applies the central-difference update to S^n itself (an interior node has
// one slot and one chunk; a boundary node is updated identically by every chunk that
// touches it); the owner stores S^{n+1}.  The update uses explicitly rounded
// operations, so every chunk obtains the same bits.  After the last step of a call
// k_finalize_nodes completes S^N.
// ---------------------------------------------------------------------------
struct FusedArgs {
  DevPlan P;
  double* u_cur[3];
  double* v_cur[3];
  double* u_prv[3];
  double* v_prv[3];
  const float* halo_prv[3];
  float* halo_cur[3];
  const float* mass;
  const double* d0;
  const float* d0f;  // d0 rounded to FP32 (wall screening)
  unsigned char* contact;
  float* acc[3];
  float4* sig_a;
  float2* sig_b;
  float* epbar;
  double* chunk_work;
  unsigned int* status;
  int state_final;  // every node already holds S^n in the cur buffer (first step of a call)
  int store_acc;
  // batched solves (k_step<..., BATCH = true>): per-instance parameters and step counts;
  // the global step is *step_ctr + step_off.  An instance steps while step < nsteps,
  // completes its nodes at step == nsteps and idles afterwards.
  const ElemParams* inst_ep;
  const NodeParams* inst_np;
  const int* inst_nsteps;
  const int* step_ctr;
  int step_off;
};

// Per-chunk view of the step: parameters, whether to step, finalise only, or idle.
struct ChunkStep {
  ElemParams ep;
  NodeParams np;
  int state_final;
  int mode;  // 0 step, 1 complete the nodes only, 2 idle
};

template <bool BATCH>
__device__ __forceinline__ ChunkStep chunk_step(const FusedArgs& A, const ChunkInfo& ch,
                                                const ElemParams& ep, const NodeParams& np) {
  ChunkStep c;
  if (!BATCH) {
    c.ep = ep;
    c.np = np;
    c.state_final = A.state_final;
    c.mode = 0;
    return c;
  }
  const int k = *A.step_ctr + A.step_off;
  const int n = A.inst_nsteps[ch.inst];
  c.ep = A.inst_ep[ch.inst];
  c.np = A.inst_np[ch.inst];
  c.state_final = k == 0;
  c.mode = k < n ? 0 : (k == n ? 1 : 2);
  return c;
}

// One node's central-difference update from its total internal force f.
// u, v: in S^n, out S^{n+1}; a: the acceleration applied.  Rounding is explicit (no
// contraction freedom), so every chunk that updates the same boundary node gets the
// same bits.  FP64 work is 6 FMAs per node: u + dt v and v + dt a.  The acceleration
// -f/m + g is formed in FP32 (as accurate as f); the wall distance is screened in FP32
// with a margin above its worst rounding error and only evaluated in FP64 near or
// inside the wall.
__device__ __forceinline__ void node_step(const NodeParams& p, float fx, float fy, float fz, float m,
                                          float d0f, const double* d0, int g, double (&u)[3],
                                          double (&v)[3], float (&a)[3], bool& in_contact,
                                          float (&uf_out)[3], float (&vf_out)[3]) {
  const float rm = __frcp_rn(m);
  a[0] = __fadd_rn(__fmul_rn(-fx, rm), p.gf[0]);
  a[1] = __fadd_rn(__fmul_rn(-fy, rm), p.gf[1]);
  a[2] = __fadd_rn(__fmul_rn(-fz, rm), p.gf[2]);
  double un[3];
  float uf[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    un[k] = __fma_rn(p.dt, v[k], u[k]);
    uf[k] = f64_to_f32(un[k]);
  }
  // |d32 - d| <= 2^-22 (|d0| + |u|_1) for |n_k| <= 1; 1e-6 (1 + ...) covers it
  const float d32 = __fadd_rn(d0f, __fadd_rn(__fmul_rn(p.nf[0], uf[0]),
                                  __fadd_rn(__fmul_rn(p.nf[1], uf[1]), __fmul_rn(p.nf[2], uf[2]))));
  const float margin = 1e-6f * (1.f + fabsf(d0f) + fabsf(uf[0]) + fabsf(uf[1]) + fabsf(uf[2]));
  in_contact = false;
  double ad[3] = {f32_to_f64(a[0]), f32_to_f64(a[1]), f32_to_f64(a[2])};
  if (!(d32 > margin)) {
    const double d = __fma_rn(p.wall_n[2], un[2], __fma_rn(p.wall_n[1], un[1],
                              __fma_rn(p.wall_n[0], un[0], d0[g])));
    if (d < 0.0) {
      in_contact = true;
      const double c = __ddiv_rn(__dmul_rn(-d, p.wall_k), (double)m);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        ad[k] = __fma_rn(c, p.wall_n[k], ad[k]);
        a[k] = f64_to_f32(ad[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    v[k] = __fma_rn(p.dt, ad[k], v[k]);
    u[k] = un[k];
    uf_out[k] = uf[k];
    vf_out[k] = f64_to_f32(v[k]);
  }
}

__device__ __forceinline__ void store_node(const FusedArgs& A, double* const (&uo)[3],
                                           double* const (&vo)[3], int g, const double (&u)[3],
                                           const double (&v)[3], const float (&vf)[3],
                                           const float (&a)[3], bool in_contact, bool store_acc,
                                           unsigned char old) {
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    uo[k][g] = u[k];
    vo[k][g] = v[k];
    finite = finite && isfinite(vf[k]);
    if (store_acc) A.acc[k][g] = a[k];
  }
  if (!finite) atomicOr(A.status, (unsigned)ST_NONFINITE);
  const unsigned char flag = in_contact ? 3 : (old & 2);
  if (flag != old) A.contact[g] = flag;
}

// S^n of node g from S^{n-1} (prv buffer) and the halo of step n-1: the sum of its
// slots [s0, s1) in fixed order, then the update.  Every chunk touching g computes the same bits.
__device__ __forceinline__ void complete_node(const FusedArgs& A, const NodeParams& np, int g,
                                              int s0, int s1, double (&u)[3], double (&v)[3],
                                              float (&a)[3], bool& hit, float (&uf)[3],
                                              float (&vf)[3]) {
  float fx = 0.f, fy = 0.f, fz = 0.f;
  for (int s = s0; s < s1; s++) {
    fx = __fadd_rn(fx, A.halo_prv[0][s]);
    fy = __fadd_rn(fy, A.halo_prv[1][s]);
    fz = __fadd_rn(fz, A.halo_prv[2][s]);
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    u[k] = A.u_prv[k][g];
    v[k] = A.v_prv[k][g];
  }
  node_step(np, fx, fy, fz, A.mass[g], A.d0f[g], A.d0, g, u, v, a, hit, uf, vf);
}

// Shared-memory node records of the fused kernels: p0 = (x, du_x, y, du_y),
// p1 = (z, du_z), acc = (f_x, f_y, f_z, -); 40 bytes per local node.  Each coordinate
// and its increment are adjacent, so a record loads as three (x_c, du_c) register
// pairs, the operand shape of the packed FP32 instructions (fma.rn.f32x2).
struct Tile {
  float4* p0;
  float2* p1;
  float4* acc;
};

__device__ __forceinline__ void store_record(const Tile& T, int l, float x, float y, float z,
                                             float dx, float dy, float dz) {
  T.p0[l] = make_float4(x, dx, y, dy);
  T.p1[l] = make_float2(z, dz);
}

// (x_c, du_c) of local node l for c = 0, 1, 2
__device__ __forceinline__ void load_pairs(const Tile& T, int l, float2 (&p)[3]) {
  const float4 q0 = T.p0[l];
  p[0] = make_float2(q0.x, q0.y);
  p[1] = make_float2(q0.z, q0.w);
  p[2] = T.p1[l];
}

// Zero local node l's force accumulator and keep the node's halo slot in this chunk in
// its fourth lane (as int bits; the element loops add to x, y, z only), so that the
// epilogue writes the partial forces without a dependent load.
__device__ __forceinline__ void init_acc(const Tile& T, const ChunkInfo& ch, const DevPlan& P,
                                         int l) {
  const int s = l < ch.n_int ? ch.slot_begin + l : P.local_slot[ch.local_begin + l];
  T.acc[l] = make_float4(0.f, 0.f, 0.f, __int_as_float(s));
}

__device__ __forceinline__ Tile make_tile(float* sm, int L) {
  Tile t;
  t.p0 = reinterpret_cast<float4*>(sm);
  t.p1 = reinterpret_cast<float2*>(t.p0 + L);
  t.acc = reinterpret_cast<float4*>(t.p1 + ((L + 1) & ~1));
  return t;
}

// Stage S^n of every local node of the chunk in shared memory (x relative to the
// chunk origin, dt v): completed from S^{n-1} and the previous halo (the owner stores
// it), or read as it is on the first step of a call.  All of a node's loads (slot
// range, halo slots, state, mass, wall distance, contact flag, reference position) are
// issued before its update and stores.
template <int BS>
__device__ __forceinline__ void stage_nodes(const FusedArgs& A, const ElemParams& ep,
                                            const NodeParams& np, const ChunkInfo& ch,
                                            int state_final, const Tile& T, int tid) {
  const DevPlan& P = A.P;
  const int L = ch.n_local;
  for (int l = tid; l < L; l += BS) {
    const int lb = ch.local_begin + l;
    const bool own = l < ch.n_own;
    const int g = own ? ch.own_begin + l : P.local_gid[lb];
    float x0[3], uf[3], vf[3];
#pragma unroll
    for (int k = 0; k < 3; k++) x0[k] = P.local_x0[k * (size_t)P.Lt + lb];
    if (state_final) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        uf[k] = f64_to_f32(A.u_cur[k][g]);
        vf[k] = f64_to_f32(A.v_cur[k][g]);
      }
    } else {
      // interior nodes: one slot at a known position; others: their node's slot range
      int s0, s1;
      if (l < ch.n_int) {
        s0 = ch.slot_begin + l;
        s1 = s0 + 1;
      } else {
        const int2 r = P.local_srow[lb];
        s0 = r.x;
        s1 = r.y;
      }
      // slot sum in slot order starting from 0 (s1 > s0: the node's slot in this chunk)
      const bool two = s1 > s0 + 1;
      float f[3];
      double u[3], v[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float h0 = A.halo_prv[k][s0];
        const float h1 = two ? A.halo_prv[k][s0 + 1] : 0.f;
        f[k] = __fadd_rn(0.f, h0);
        if (two) f[k] = __fadd_rn(f[k], h1);
        u[k] = A.u_prv[k][g];
        v[k] = A.v_prv[k][g];
      }
      const float m = A.mass[g], d0f = A.d0f[g];
      const unsigned char ct = A.contact[g];
      for (int sl = s0 + 2; sl < s1; sl++) {
#pragma unroll
        for (int k = 0; k < 3; k++) f[k] = __fadd_rn(f[k], A.halo_prv[k][sl]);
      }
      float a[3];
      bool hit;
      node_step(np, f[0], f[1], f[2], m, d0f, A.d0, g, u, v, a, hit, uf, vf);
      if (own) store_node(A, A.u_cur, A.v_cur, g, u, v, vf, a, hit, false, ct);
    }
    store_record(T, l, x0[0] + uf[0], x0[1] + uf[1], x0[2] + uf[2], ep.dt * vf[0], ep.dt * vf[1],
                 ep.dt * vf[2]);
    init_acc(T, ch, P, l);
  }
}

// stage_nodes with K nodes per thread in flight: the loads of K nodes are issued before
// the first of their updates (for kernels with registers to spare during the staging).
template <int BS, int K>
__device__ __forceinline__ void stage_nodes_k(const FusedArgs& A, const ElemParams& ep,
                                              const NodeParams& np, const ChunkInfo& ch,
                                              int state_final, const Tile& T, int tid) {
  if (K == 1 || state_final) {
    stage_nodes<BS>(A, ep, np, ch, state_final, T, tid);
    return;
  }
  const DevPlan& P = A.P;
  const int L = ch.n_local;
  for (int l0 = tid; l0 < L; l0 += K * BS) {
    int g[K], s0[K], s1[K];
#pragma unroll
    for (int j = 0; j < K; j++) {
      const int l = min(l0 + j * BS, L - 1);  // past the end: repeat the last node, unused
      const int lb = ch.local_begin + l;
      g[j] = l < ch.n_own ? ch.own_begin + l : P.local_gid[lb];
      if (l < ch.n_int) {
        s0[j] = ch.slot_begin + l;
        s1[j] = s0[j] + 1;
      } else {
        const int2 r = P.local_srow[lb];
        s0[j] = r.x;
        s1[j] = r.y;
      }
    }
    float f[K][3], m[K], d0f[K], x0[K][3];
    double u[K][3], v[K][3];
    unsigned char ct[K];
#pragma unroll
    for (int j = 0; j < K; j++) {
      const size_t lb = ch.local_begin + min(l0 + j * BS, L - 1);
      const bool two = s1[j] > s0[j] + 1;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float h0 = A.halo_prv[k][s0[j]];
        const float h1 = two ? A.halo_prv[k][s0[j] + 1] : 0.f;
        f[j][k] = __fadd_rn(0.f, h0);
        if (two) f[j][k] = __fadd_rn(f[j][k], h1);
        u[j][k] = A.u_prv[k][g[j]];
        v[j][k] = A.v_prv[k][g[j]];
        x0[j][k] = P.local_x0[k * (size_t)P.Lt + lb];
      }
      m[j] = A.mass[g[j]];
      d0f[j] = A.d0f[g[j]];
      ct[j] = A.contact[g[j]];
    }
#pragma unroll
    for (int j = 0; j < K; j++)
      for (int sl = s0[j] + 2; sl < s1[j]; sl++) {
#pragma unroll
        for (int k = 0; k < 3; k++) f[j][k] = __fadd_rn(f[j][k], A.halo_prv[k][sl]);
      }
#pragma unroll
    for (int j = 0; j < K; j++) {
      const int l = l0 + j * BS;
      if (l >= L) break;
      float a[3], uf[3], vf[3];
      bool hit;
      node_step(np, f[j][0], f[j][1], f[j][2], m[j], d0f[j], A.d0, g[j], u[j], v[j], a, hit, uf,
                vf);
      if (l < ch.n_own) store_node(A, A.u_cur, A.v_cur, g[j], u[j], v[j], vf, a, hit, false, ct[j]);
      store_record(T, l, x0[j][0] + uf[0], x0[j][1] + uf[1], x0[j][2] + uf[2], ep.dt * vf[0],
                   ep.dt * vf[1], ep.dt * vf[2]);
      init_acc(T, ch, P, l);
    }
  }
}

// Every local node's partial force of this step to its slot in the halo (the slot kept in
// the accumulator's fourth lane by init_acc).
template <int BS>
__device__ __forceinline__ void node_epilogue(const FusedArgs& A, const ChunkInfo& ch,
                                              const Tile& T, int tid) {
  const int L = ch.n_local;
#pragma unroll 4
  for (int l = tid; l < L; l += BS) {
    const float4 f = T.acc[l];
    const int s = __float_as_int(f.w);
    A.halo_cur[0][s] = f.x;
    A.halo_cur[1][s] = f.y;
    A.halo_cur[2][s] = f.z;
  }
}

// The CTA's internal and plastic work of this step added to chunk c's running sums by
// reductions at L2 (no round trip before the CTA's next barrier).  Only one CTA at a time
// updates a chunk's sums, in step order, so every addition is the one
// sums = sums + (double)t of the step order, and the sums' bits do not depend on timing.
template <int BS>
__device__ __forceinline__ void add_chunk_work(const FusedArgs& A, int c, float wint, float wp,
                                               float* red) {
  const float t0 = block_sum<BS>(wint, red);
  const float t1 = block_sum<BS>(wp, red);
  if (threadIdx.x == 0) {
    double* cw = A.chunk_work + 4 * (size_t)c;
    atomicAdd(cw, (double)t0);
    atomicAdd(cw + 1, (double)t1);
  }
}

// Fused step, one thread per element (tet4, and the tet10 reference variant).
template <int NPE, int MODE, int BS, bool BATCH = false>
__global__ void __launch_bounds__(BS) k_step(FusedArgs A, ElemParams ep_arg, NodeParams np_arg) {
  extern __shared__ float sm[];
  const DevPlan& P = A.P;
  const ChunkInfo ch = P.chunks[blockIdx.x];
  const ChunkStep cs = chunk_step<BATCH>(A, ch, ep_arg, np_arg);
  if (cs.mode == 2) return;
  const ElemParams& ep = cs.ep;
  const NodeParams& np = cs.np;
  const int L = ch.n_local;
  const Tile T = make_tile(sm, L);
  __shared__ float red[BS / 32];

  stage_nodes<BS>(A, ep, np, ch, cs.state_final, T, threadIdx.x);
  if (cs.mode == 1) return;
  __syncthreads();

  DevState S;
  S.sig_a = A.sig_a;
  S.sig_b = A.sig_b;
  S.epbar = A.epbar;
  S.status = A.status;
  float wint = 0.f, wp = 0.f, vol = 0.f;
  const int E = P.E;
  for (int w = ch.elem_begin; w < ch.elem_end; w += BS) {
    const int e = w + threadIdx.x;
    const bool act = e < ch.elem_end;
    int col = -1;
    int ln[NPE];
    float f[NPE][3];
    if (act) {
      col = P.color[e];
      float x[NPE][3], du[NPE][3];
#pragma unroll
      for (int a = 0; a < NPE; a++) {
        ln[a] = P.conn_local[(size_t)a * E + e];
        float2 pr[3];
        load_pairs(T, ln[a], pr);
#pragma unroll
        for (int c = 0; c < 3; c++) {
          x[a][c] = pr[c].x;
          du[a][c] = pr[c].y;
        }
      }
      element_force<NPE, MODE>(ep, S, e, E, x, du, f, wint, wp, vol);
    }
    const int c0 = P.color[w];
    const int c1 = P.color[min(w + BS, ch.elem_end) - 1];
    for (int k = c0; k <= c1; k++) {
      __syncthreads();
      if (col == k) {
#pragma unroll
        for (int a = 0; a < NPE; a++) {
          float4 t = T.acc[ln[a]];
          t.x += f[a][0];
          t.y += f[a][1];
          t.z += f[a][2];
          T.acc[ln[a]] = t;
        }
      }
    }
  }
  __syncthreads();
  node_epilogue<BS>(A, ch, T, threadIdx.x);
  if (ep.accum_energy) add_chunk_work<BS>(A, blockIdx.x, wint, wp, red);
}

// ---------------------------------------------------------------------------
// tet10 with one lane per Gauss point (lanes 4k..4k+3 of a warp share an element).
//
// With barycentrics L = (xi, eta, 1-xi-eta-zeta, zeta) at the lane's point and
// A_c = 4 L_c, the shape-function gradients are G_0 = (A0-1, 0, 0), G_1 = (0, A1-1, 0),
// G_2 = -(A2-1)(1,1,1), G_3 = (0, 0, A3-1), G_4 = (A1, A0, 0),
// G_5 = (-A1, A2-A1, -A1), G_6 = (A2-A0, -A0, -A0), G_7 = (A3, 0, A0),
// G_8 = (0, A3, A1), G_9 = (-A3, -A3, A2-A3).  J = sum_i x_i G_i^T and grad du are
// built from nodes streamed out of shared memory; the lane's Gauss-point force
// contributions P G_i are summed over the four lanes by an xor butterfly (fixed
// order, so the result is bitwise reproducible).
// ---------------------------------------------------------------------------
struct Tet10QP {
  float A0, A1, A2, A3;
};

__device__ __forceinline__ Tet10QP tet10_qp(int q) {
  const float a = 0.58541019662496845f, b = 0.13819660112501052f;
  Tet10QP t;
  t.A0 = 4.f * (q == 1 ? a : b);
  t.A1 = 4.f * (q == 2 ? a : b);
  t.A2 = 4.f * (q == 0 ? a : b);
  t.A3 = 4.f * (q == 3 ? a : b);
  return t;
}

// c[j] += x * G_i[j] for node i of the tet10 at this lane's point.
template <int I>
__device__ __forceinline__ void tet10_grad_acc(const Tet10QP& t, float x, float (&c)[3]) {
  if (I == 0) c[0] = fmaf(t.A0 - 1.f, x, c[0]);
  if (I == 1) c[1] = fmaf(t.A1 - 1.f, x, c[1]);
  if (I == 2) {
    const float g = (1.f - t.A2) * x;
    c[0] += g; c[1] += g; c[2] += g;
  }
  if (I == 3) c[2] = fmaf(t.A3 - 1.f, x, c[2]);
  if (I == 4) { c[0] = fmaf(t.A1, x, c[0]); c[1] = fmaf(t.A0, x, c[1]); }
  if (I == 5) { c[0] = fmaf(-t.A1, x, c[0]); c[1] = fmaf(t.A2 - t.A1, x, c[1]); c[2] = fmaf(-t.A1, x, c[2]); }
  if (I == 6) { c[0] = fmaf(t.A2 - t.A0, x, c[0]); c[1] = fmaf(-t.A0, x, c[1]); c[2] = fmaf(-t.A0, x, c[2]); }
  if (I == 7) { c[0] = fmaf(t.A3, x, c[0]); c[2] = fmaf(t.A0, x, c[2]); }
  if (I == 8) { c[1] = fmaf(t.A3, x, c[1]); c[2] = fmaf(t.A1, x, c[2]); }
  if (I == 9) { c[0] = fmaf(-t.A3, x, c[0]); c[1] = fmaf(-t.A3, x, c[1]); c[2] = fmaf(t.A2 - t.A3, x, c[2]); }
}

// f = P G_i (row a of P times the gradient of node i)
template <int I>
__device__ __forceinline__ float tet10_force(const Tet10QP& t, const float* Pa) {
  if (I == 0) return (t.A0 - 1.f) * Pa[0];
  if (I == 1) return (t.A1 - 1.f) * Pa[1];
  if (I == 2) return (1.f - t.A2) * (Pa[0] + Pa[1] + Pa[2]);
  if (I == 3) return (t.A3 - 1.f) * Pa[2];
  if (I == 4) return fmaf(t.A1, Pa[0], t.A0 * Pa[1]);
  if (I == 5) return fmaf(-t.A1, Pa[0], fmaf(t.A2 - t.A1, Pa[1], -t.A1 * Pa[2]));
  if (I == 6) return fmaf(t.A2 - t.A0, Pa[0], -t.A0 * (Pa[1] + Pa[2]));
  if (I == 7) return fmaf(t.A3, Pa[0], t.A0 * Pa[2]);
  if (I == 8) return fmaf(t.A3, Pa[1], t.A1 * Pa[2]);
  return fmaf(-t.A3, Pa[0] + Pa[1], (t.A2 - t.A3) * Pa[2]);
}

// Packed (FP32 pair) form of tet10_grad_acc: c[j] += G_I[j] * (x, du) for one
// coordinate's (position, increment) pair, two results per instruction
// (fma.rn.f32x2 / add / mul, sm_100 and later).
__device__ __forceinline__ float2 bcast(float a) { return make_float2(a, a); }

template <int I>
__device__ __forceinline__ void tet10_grad_acc2(const Tet10QP& t, float2 x, float2* c) {
  if (I == 0) c[0] = __ffma2_rn(bcast(t.A0 - 1.f), x, c[0]);
  if (I == 1) c[1] = __ffma2_rn(bcast(t.A1 - 1.f), x, c[1]);
  if (I == 2) {
    const float2 g = __fmul2_rn(bcast(1.f - t.A2), x);
    c[0] = __fadd2_rn(c[0], g);
    c[1] = __fadd2_rn(c[1], g);
    c[2] = __fadd2_rn(c[2], g);
  }
  if (I == 3) c[2] = __ffma2_rn(bcast(t.A3 - 1.f), x, c[2]);
  if (I == 4) {
    c[0] = __ffma2_rn(bcast(t.A1), x, c[0]);
    c[1] = __ffma2_rn(bcast(t.A0), x, c[1]);
  }
  if (I == 5) {
    c[0] = __ffma2_rn(bcast(-t.A1), x, c[0]);
    c[1] = __ffma2_rn(bcast(t.A2 - t.A1), x, c[1]);
    c[2] = __ffma2_rn(bcast(-t.A1), x, c[2]);
  }
  if (I == 6) {
    c[0] = __ffma2_rn(bcast(t.A2 - t.A0), x, c[0]);
    c[1] = __ffma2_rn(bcast(-t.A0), x, c[1]);
    c[2] = __ffma2_rn(bcast(-t.A0), x, c[2]);
  }
  if (I == 7) {
    c[0] = __ffma2_rn(bcast(t.A3), x, c[0]);
    c[2] = __ffma2_rn(bcast(t.A0), x, c[2]);
  }
  if (I == 8) {
    c[1] = __ffma2_rn(bcast(t.A3), x, c[1]);
    c[2] = __ffma2_rn(bcast(t.A1), x, c[2]);
  }
  if (I == 9) {
    c[0] = __ffma2_rn(bcast(-t.A3), x, c[0]);
    c[1] = __ffma2_rn(bcast(-t.A3), x, c[1]);
    c[2] = __ffma2_rn(bcast(t.A2 - t.A3), x, c[2]);
  }
}

// JG[3a + j] = (J, grad du)[a][j] += G_I[j] * (x_a, du_a) for local node l
template <int I>
__device__ __forceinline__ void tet10_gather(const Tet10QP& t, const Tile& T, int l, float2 (&JG)[9]) {
  float2 p[3];
  load_pairs(T, l, p);
#pragma unroll
  for (int a = 0; a < 3; a++) tet10_grad_acc2<I>(t, p[a], &JG[3 * a]);
}

// Force component c of node I at this lane's point (I < 0: none).
template <int I>
__device__ __forceinline__ float tet10_fc(const Tet10QP& t, const float (&Pm)[9], int c) {
  if (I < 0) return 0.f;
  return tet10_force<(I < 0 ? 0 : I)>(t, &Pm[3 * c]);
}

// Sum over the 4 lanes of an element (its 4 points) of the forces of the nodes lane q
// owns, delivered to lane q only: R[0..2] node q, R[3..5] node q + 4, R[6..8] node
// q + 8 (q < 2).  Two butterfly levels: xor 2 leaves lanes 0, 1 with nodes
// {0,4,8,1,5,9} and lanes 2, 3 with {2,6,3,7}; xor 1 splits each pair.
template <int K>
__device__ __forceinline__ void tet10_rs_slot(const Tet10QP& t, const float (&Pm)[9], bool lo,
                                              bool even, float (&R)[9]) {
  constexpr int r = K / 3, c = K % 3;
  constexpr int L0 = r == 0 ? 0 : r == 1 ? 4 : 8;
  constexpr int L1 = r == 0 ? 1 : r == 1 ? 5 : 9;
  constexpr int H0 = r == 0 ? 2 : r == 1 ? 6 : -1;
  constexpr int H1 = r == 0 ? 3 : r == 1 ? 7 : -1;
  const float a0 = tet10_fc<L0>(t, Pm, c), a1 = tet10_fc<L1>(t, Pm, c);
  float m0, m1;
  if (H0 >= 0) {
    const float b0 = tet10_fc<H0>(t, Pm, c), b1 = tet10_fc<H1>(t, Pm, c);
    m0 = (lo ? a0 : b0) + __shfl_xor_sync(0xffffffffu, lo ? b0 : a0, 2);
    m1 = (lo ? a1 : b1) + __shfl_xor_sync(0xffffffffu, lo ? b1 : a1, 2);
  } else {
    m0 = a0 + __shfl_xor_sync(0xffffffffu, a0, 2);
    m1 = a1 + __shfl_xor_sync(0xffffffffu, a1, 2);
  }
  R[K] = (even ? m0 : m1) + __shfl_xor_sync(0xffffffffu, even ? m1 : m0, 1);
}

// Element loop of one chunk by the CTA's BS threads (4 lanes per element, colours
// applied in order between barriers) into the tile's force accumulators; this thread's
// internal and plastic work in wint, wp.  CG: the stored stress and plastic strain are
// read through L2 only (the persistent task kernel, where another SM may have written
// them last).  PF: the next window's connectivity, stored stress and colours are loaded
// before the current window's colour loop (where few registers are live), so that their
// round trip overlaps the accumulation instead of stalling the next window's gather.
template <int MODE, int BS, bool CG, bool PF>
__device__ __forceinline__ void qp10_element_loop(const FusedArgs& A, const ElemParams& ep,
                                                  const ChunkInfo& ch, const Tile& T, int tid,
                                                  float& wint, float& wp) {
  const DevPlan& P = A.P;
  const int q = tid & 3;
  const Tet10QP t = tet10_qp(q);
  constexpr float W = 1.0f / 24.0f;
  const int E = P.E;
  wint = 0.f;
  wp = 0.f;
  constexpr int EPW = BS / 4;  // elements per window
  // window loads: connectivity, stored stress and plastic strain of this lane's point,
  // the element's colour and the window's first and last colours
  int ln[10];
  float4 s4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 s2 = make_float2(0.f, 0.f);
  float ep0 = 0.f;
  int wcol = -1, wc0 = 0, wc1 = -1;
  auto window_loads = [&](int w) {
    const int e = w + (tid >> 2);
    const bool act = e < ch.elem_end;
    const int ee = act ? e : ch.elem_begin;  // inactive lanes shadow a valid element
#pragma unroll
    for (int a = 0; a < 10; a++) ln[a] = P.conn_local[(size_t)a * E + ee];
    const size_t qi = (size_t)ee * 4 + q;
    if (MODE == EM_J2) {
      s4 = CG ? __ldcg(A.sig_a + qi) : A.sig_a[qi];
      s2 = CG ? __ldcg(A.sig_b + qi) : A.sig_b[qi];
      ep0 = CG ? __ldcg(A.epbar + qi) : A.epbar[qi];
    }
    wcol = act ? P.color[e] : -1;
    wc0 = P.color[w];
    wc1 = P.color[min(w + EPW, ch.elem_end) - 1];
  };
  if (PF && ch.elem_begin < ch.elem_end) window_loads(ch.elem_begin);
  for (int w = ch.elem_begin; w < ch.elem_end; w += EPW) {
    const int e = w + (tid >> 2);
    const bool act = e < ch.elem_end;
    const int ee = act ? e : ch.elem_begin;
    const size_t qi = (size_t)ee * 4 + q;
    if (!PF) window_loads(w);
    float2 JG[9];
#pragma unroll
    for (int k = 0; k < 9; k++) JG[k] = make_float2(0.f, 0.f);
    tet10_gather<0>(t, T, ln[0], JG);
    tet10_gather<1>(t, T, ln[1], JG);
    tet10_gather<2>(t, T, ln[2], JG);
    tet10_gather<3>(t, T, ln[3], JG);
    tet10_gather<4>(t, T, ln[4], JG);
    tet10_gather<5>(t, T, ln[5], JG);
    tet10_gather<6>(t, T, ln[6], JG);
    tet10_gather<7>(t, T, ln[7], JG);
    tet10_gather<8>(t, T, ln[8], JG);
    tet10_gather<9>(t, T, ln[9], JG);
    float J[9], Gu[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
      J[k] = JG[k].x;
      Gu[k] = JG[k].y;
    }
    float Ji[9];
    const float detJ = inv3f(J, Ji);
    if (act && !(detJ > 0.f)) atomicOr(A.status, (unsigned)ST_DEGENERATE);
    const float wd = act ? W * detJ : 0.f;
    float Lg[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++)
        Lg[3 * a + b] = Gu[3 * a + 0] * Ji[0 * 3 + b] + Gu[3 * a + 1] * Ji[1 * 3 + b] +
                        Gu[3 * a + 2] * Ji[2 * 3 + b];
    const float de[6] = {Lg[0], Lg[4], Lg[8], Lg[1] + Lg[3], Lg[5] + Lg[7], Lg[2] + Lg[6]};
    const float tr = de[0] + de[1] + de[2];
    const float s0[6] = {s4.x, s4.y, s4.z, s4.w, s2.x, s2.y};
    float s[6];
    s[0] = s0[0] + ep.lambda * tr + 2.f * ep.mu * de[0];
    s[1] = s0[1] + ep.lambda * tr + 2.f * ep.mu * de[1];
    s[2] = s0[2] + ep.lambda * tr + 2.f * ep.mu * de[2];
    s[3] = s0[3] + ep.mu * de[3];
    s[4] = s0[4] + ep.mu * de[4];
    s[5] = s0[5] + ep.mu * de[5];
    float epn = ep0;
    if (MODE == EM_J2) {
      j2_return(ep, s, epn);
      if (act) {
        A.sig_a[qi] = make_float4(s[0], s[1], s[2], s[3]);
        A.sig_b[qi] = make_float2(s[4], s[5]);
        A.epbar[qi] = epn;
      }
    }
    if (ep.accum_energy && act) {
      float wq = 0.f;
#pragma unroll
      for (int k = 0; k < 6; k++) wq = fmaf(s0[k] + s[k], de[k], wq);
      wint = fmaf(0.5f * wd, wq, wint);
      if (MODE == EM_J2) wp = fmaf(wd * (ep.sy0 + ep.H * epn), epn - ep0, wp);
    }
    const float Sg[9] = {s[0], s[3], s[5], s[3], s[1], s[4], s[5], s[4], s[2]};
    float Pm[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        Pm[3 * a + j] = wd * (Sg[3 * a + 0] * Ji[3 * j + 0] + Sg[3 * a + 1] * Ji[3 * j + 1] +
                              Sg[3 * a + 2] * Ji[3 * j + 2]);
    float keep[3][3];
    {
      float R[9];
      const bool lo = q < 2, even = (q & 1) == 0;
      tet10_rs_slot<0>(t, Pm, lo, even, R);
      tet10_rs_slot<1>(t, Pm, lo, even, R);
      tet10_rs_slot<2>(t, Pm, lo, even, R);
      tet10_rs_slot<3>(t, Pm, lo, even, R);
      tet10_rs_slot<4>(t, Pm, lo, even, R);
      tet10_rs_slot<5>(t, Pm, lo, even, R);
      tet10_rs_slot<6>(t, Pm, lo, even, R);
      tet10_rs_slot<7>(t, Pm, lo, even, R);
      tet10_rs_slot<8>(t, Pm, lo, even, R);
#pragma unroll
      for (int k = 0; k < 9; k++) keep[k / 3][k % 3] = R[k];
    }
    // lane q owns nodes q, q+4 and (for q < 2) q+8
    const int own0 = q == 0 ? ln[0] : q == 1 ? ln[1] : q == 2 ? ln[2] : ln[3];
    const int own1 = q == 0 ? ln[4] : q == 1 ? ln[5] : q == 2 ? ln[6] : ln[7];
    const int own2 = q == 0 ? ln[8] : ln[9];
    const int col = wcol, c0 = wc0, c1 = wc1;
    if (PF && w + EPW < ch.elem_end) window_loads(w + EPW);
    for (int k = c0; k <= c1; k++) {
      __syncthreads();
      if (col == k) {
        float4 t0 = T.acc[own0];
        t0.x += keep[0][0];
        t0.y += keep[0][1];
        t0.z += keep[0][2];
        T.acc[own0] = t0;
        float4 t1 = T.acc[own1];
        t1.x += keep[1][0];
        t1.y += keep[1][1];
        t1.z += keep[1][2];
        T.acc[own1] = t1;
        if (q < 2) {
          float4 t2 = T.acc[own2];
          t2.x += keep[2][0];
          t2.y += keep[2][1];
          t2.z += keep[2][2];
          T.acc[own2] = t2;
        }
      }
    }
  }
}

// The fused kernels' element phase: the loop, then the chunk's partial nodal forces to
// the halo and its work to chunk c's sums.
template <int MODE, int BS, bool PF>
__device__ __forceinline__ void step_qp10_elements(const FusedArgs& A, const ElemParams& ep,
                                                   const ChunkInfo& ch, const Tile& T, int tid,
                                                   int c, float* red) {
  float wint, wp;
  qp10_element_loop<MODE, BS, false, PF>(A, ep, ch, T, tid, wint, wp);
  __syncthreads();
  node_epilogue<BS>(A, ch, T, tid);
  if (ep.accum_energy) add_chunk_work<BS>(A, c, wint, wp, red);
}

// 6 CTAs of 128 threads per SM (80 registers) fit the 896-node chunk's shared tile
template <int MODE, int BS, bool BATCH = false>
__global__ void __launch_bounds__(BS, 768 / BS) k_step_qp10(FusedArgs A, ElemParams ep_arg, NodeParams np_arg) {
  extern __shared__ float sm[];
  const DevPlan& P = A.P;
  const ChunkInfo ch = P.chunks[blockIdx.x];
  const ChunkStep cs = chunk_step<BATCH>(A, ch, ep_arg, np_arg);
  if (cs.mode == 2) return;
  const Tile T = make_tile(sm, ch.n_local);
  __shared__ float red[BS / 32];

  stage_nodes<BS>(A, cs.ep, cs.np, ch, cs.state_final, T, threadIdx.x);
  if (cs.mode == 1) return;
  __syncthreads();
  step_qp10_elements<MODE, BS, true>(A, cs.ep, ch, T, threadIdx.x, blockIdx.x, red);
}

// ---------------------------------------------------------------------------
// Persistent task kernel of the four-lane tet10 step (step_kernel = 2).
//
// A call of n steps is one launch whose CTAs claim tasks from a counter, in the order
//   N(0, .);  then for j = 0 .. n-1:  E(j, .), N(j+1, .),
// each block in one task order of the chunks (reverse Cuthill-McKee on the graph of
// chunks sharing a node, so that a task's dependencies lie about one block back).
// N(j, c): chunk c completes S^j of the nodes it owns -- from S^{j-1} and the halo of step
//   j-1 exactly as the fused kernel's staging does (N(0) reads the state as it is, N(n)
//   also stores the accelerations) -- and writes each node's record (u and dt v rounded to
//   FP32) to the record buffers of parity j.
// E(j, c): chunk c stages its local nodes from those records (x = chunk-relative X0 + u,
//   the fused kernel's sum) and runs the element loop of step j, writing its halo partials
//   (parity j), stored stress and work sums.
// E(j, c) waits until every chunk owning one of c's nodes has finished N(j, .); N(j, c)
// waits until every chunk with a slot of one of c's nodes has finished E(j-1, .).  These
// waits order every reuse of the double buffers (records, halo, state) as well: E(j-2, t)
// precedes N(j-1, c) precedes E(j-1, t) precedes N(j, c) for any chunk t touching c.  Every
// dependency of a task comes earlier in the claim order and only a running CTA claims,
// so the earliest unfinished task can always proceed.  Each node is completed once (no
// ghost copies), and CTAs doing node tasks (memory and FP64 bound) share the SMs with
// CTAs doing element tasks (FP32 issue bound).  The arithmetic is the fused kernel's, so
// on the same plan the results are the same bits.
//
// Data written by other CTAs of the launch (records, halo, state, stored stress, contact
// flags) is read through L2 only (ld.global.cg), never from a possibly stale L1 line; the
// work sums are only added to (L2 reductions).  A task publishes its completion with a
// release store after the CTA's last barrier; the lanes of warp 0 read a task's
// neighbours' counters with acquire loads, one neighbour per lane.  Every wait is bounded
// in time (wait_ns, 2 s by default): past it the CTA sets ST_FLOW_TIMEOUT and the abort
// flag, and every CTA stops at its next wait.
struct FlowArgs {
  FusedArgs A[2];        // buffers of an even / odd step: state cur/prv, halo cur/prv
  float4* rec_a[2];      // per node and parity: (u_x, u_y, u_z, dt v_x) in FP32
  float2* rec_b[2];      //                       (dt v_y, dt v_z)
  // [2][C][desc_stride] ints, 16-byte aligned: kind 0 = element task, 1 = node task, by
  // position in the task order of the chunks; ChunkInfo, the chunk id at kFlowDescChunk,
  // the length of the task's dependency list at kFlowDescCount and the list from
  // kFlowDescHead (element task: the chunks owning one of its local nodes; node task:
  // the chunks holding a local entry of a node it owns)
  const int* desc;
  int desc_stride;       // a multiple of 4
  int* node_done;        // [C] last j whose N(j, c) finished (-1 before the first)
  int* elem_done;        // [C] last j whose E(j, c) finished
  int* task_ctr;
  int* abort_flag;
  int C;
  int nsteps;
  unsigned long long wait_ns;  // a wait gives up after this long without progress
  int stall_chunk;             // test hook: this chunk never publishes (-1: none)
};

constexpr unsigned long long kFlowWaitNs = 2000000000ull;  // default: 2 s without progress
constexpr int kFlowDescCount = 9;
constexpr int kFlowDescChunk = 10;
constexpr int kFlowDescHead = 12;
static_assert(sizeof(ChunkInfo) == kFlowDescCount * sizeof(int), "descriptor header layout");

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One warp: wait until ctr[dep[k]] >= target for every k < n (dep in shared memory),
// lane l polling entries l, l + 32, ... at once (one round trip to L2 when the
// dependencies are met); false on abort or timeout (the same on every lane).
__device__ __forceinline__ bool flow_wait(const FlowArgs& F, const int* ctr, const int* dep, int n,
                                          int target) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
  unsigned long long t0 = 0;
  for (int k = lane; k < n && ok; k += 32) {
    const int* p = ctr + dep[k];
    for (unsigned spins = 0; ld_acquire(p) < target; spins++) {
      if (spins >= 4) __nanosleep(128);
      if ((spins & 31u) == 31u) {
        if (*(volatile int*)F.abort_flag) {
          ok = false;
          break;
        }
        const unsigned long long t = global_ns();
        if (t0 == 0) t0 = t;
        if (t - t0 > F.wait_ns) {
          atomicOr(F.A[0].status, (unsigned)ST_FLOW_TIMEOUT);
          atomicExch(F.abort_flag, 1);
          ok = false;
          break;
        }
      }
    }
  }
  return __all_sync(0xffffffffu, ok);
}

// 16-byte asynchronous copies global -> shared (through L2), completed by cp_async_wait
// in the issuing thread.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Task t: j (the step whose state it completes or uses), position r of its chunk in the
// task order, element or node task.  Order: N(0, .) for every chunk, then per step j the
// element tasks E(j, .) and the node tasks N(j + 1, .), each block in the task order of
// the chunks.
__device__ __forceinline__ void flow_decode(int t, int C, int& j, int& r, bool& elem) {
  if (t < C) {
    j = 0;
    r = t;
    elem = false;
  } else {
    const int q = (t - C) % (2 * C);
    j = (t - C) / (2 * C);
    elem = q < C;
    r = elem ? q : q - C;
    if (!elem) j++;
  }
}

// One warp: copy task t's descriptor into buf (one commit group).
__device__ __forceinline__ void flow_fetch(const FlowArgs& F, int t, int* buf) {
  int j, r;
  bool elem;
  flow_decode(t, F.C, j, r, elem);
  const int* src = F.desc + ((size_t)(elem ? 0 : F.C) + r) * F.desc_stride;
  for (int k = threadIdx.x & 31; 4 * k < F.desc_stride; k += 32) cp_async16(buf + 4 * k, src + 4 * k);
  cp_async_commit();
}

// One thread after the CTA's writes and a barrier: publish ctr[c] = j (the release
// store orders the CTA's writes, which the barrier made visible to this thread, before it).
__device__ __forceinline__ void flow_publish(int* ctr, int c, int j) { st_release(ctr + c, j); }

// N(j, c): S^j of the nodes chunk c owns and their records, one node per thread at a
// time (two in flight leave the element loop of the same kernel too few registers for
// its window prefetch, which gains more); every node's arithmetic is the fused kernel's
// staging.
template <int BS>
__device__ __forceinline__ void flow_nodes(const FlowArgs& F, const ElemParams& ep,
                                           const NodeParams& np, const ChunkInfo& ch, int j) {
  constexpr int KN = 1;
  const FusedArgs& A = F.A[j & 1];
  const DevPlan& P = A.P;
  float4* ra = F.rec_a[j & 1];
  float2* rb = F.rec_b[j & 1];
  const bool last = j == F.nsteps;
  for (int l0 = threadIdx.x; l0 < ch.n_own; l0 += KN * BS) {
    float uf[KN][3], vf[KN][3];
    if (j == 0) {
#pragma unroll
      for (int q = 0; q < KN; q++) {
        const int g = ch.own_begin + min(l0 + q * BS, ch.n_own - 1);
#pragma unroll
        for (int k = 0; k < 3; k++) {
          uf[q][k] = f64_to_f32(__ldcg(A.u_cur[k] + g));
          vf[q][k] = f64_to_f32(__ldcg(A.v_cur[k] + g));
        }
      }
    } else {
      // past the end: repeat the last owned node (loads only, results unused)
      int g[KN], s0[KN], s1[KN];
#pragma unroll
      for (int q = 0; q < KN; q++) {
        const int l = min(l0 + q * BS, ch.n_own - 1);
        g[q] = ch.own_begin + l;
        if (l < ch.n_int) {
          s0[q] = ch.slot_begin + l;
          s1[q] = s0[q] + 1;
        } else {
          const int2 r = P.local_srow[ch.local_begin + l];
          s0[q] = r.x;
          s1[q] = r.y;
        }
      }
      float f[KN][3], m[KN], d0f[KN];
      double u[KN][3], v[KN][3];
      unsigned char ct[KN];
#pragma unroll
      for (int q = 0; q < KN; q++) {
        const bool two = s1[q] > s0[q] + 1;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const float h0 = __ldcg(A.halo_prv[k] + s0[q]);
          const float h1 = two ? __ldcg(A.halo_prv[k] + s0[q] + 1) : 0.f;
          f[q][k] = __fadd_rn(0.f, h0);
          if (two) f[q][k] = __fadd_rn(f[q][k], h1);
          u[q][k] = __ldcg(A.u_prv[k] + g[q]);
          v[q][k] = __ldcg(A.v_prv[k] + g[q]);
        }
        m[q] = A.mass[g[q]];
        d0f[q] = A.d0f[g[q]];
        ct[q] = __ldcg(A.contact + g[q]);
      }
#pragma unroll
      for (int q = 0; q < KN; q++)
        for (int sl = s0[q] + 2; sl < s1[q]; sl++) {
#pragma unroll
          for (int k = 0; k < 3; k++) f[q][k] = __fadd_rn(f[q][k], __ldcg(A.halo_prv[k] + sl));
        }
#pragma unroll
      for (int q = 0; q < KN; q++) {
        if (l0 + q * BS >= ch.n_own) break;
        float a[3];
        bool hit;
        node_step(np, f[q][0], f[q][1], f[q][2], m[q], d0f[q], A.d0, g[q], u[q], v[q], a, hit,
                  uf[q], vf[q]);
        store_node(A, A.u_cur, A.v_cur, g[q], u[q], v[q], vf[q], a, hit, last, ct[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < KN; q++) {
      const int l = l0 + q * BS;
      if (l >= ch.n_own) break;
      const int g = ch.own_begin + l;
      ra[g] = make_float4(uf[q][0], uf[q][1], uf[q][2], ep.dt * vf[q][0]);
      rb[g] = make_float2(ep.dt * vf[q][1], ep.dt * vf[q][2]);
    }
  }
}

// E(j, c): the chunk's local nodes from the records of step j into the tile, KS nodes
// per thread in flight (their index, record and reference-position loads issued before
// the first shared-memory store).
template <int BS>
__device__ __forceinline__ void flow_stage(const FlowArgs& F, const ChunkInfo& ch, const Tile& T,
                                           int j) {
  constexpr int KS = 2;
  const DevPlan& P = F.A[0].P;
  const float4* ra = F.rec_a[j & 1];
  const float2* rb = F.rec_b[j & 1];
  for (int l0 = threadIdx.x; l0 < ch.n_local; l0 += KS * BS) {
    int lb[KS], g[KS], sl[KS];
#pragma unroll
    for (int q = 0; q < KS; q++) {
      const int l = min(l0 + q * BS, ch.n_local - 1);
      lb[q] = ch.local_begin + l;
      g[q] = l < ch.n_own ? ch.own_begin + l : P.local_gid[lb[q]];
      sl[q] = l < ch.n_int ? ch.slot_begin + l : P.local_slot[lb[q]];
    }
    float4 r0[KS];
    float2 r1[KS];
    float x0[KS][3];
#pragma unroll
    for (int q = 0; q < KS; q++) {
      r0[q] = __ldcg(ra + g[q]);
      r1[q] = __ldcg(rb + g[q]);
#pragma unroll
      for (int k = 0; k < 3; k++) x0[q][k] = P.local_x0[k * (size_t)P.Lt + lb[q]];
    }
#pragma unroll
    for (int q = 0; q < KS; q++) {
      const int l = l0 + q * BS;
      if (l < ch.n_local) {
        store_record(T, l, x0[q][0] + r0[q].x, x0[q][1] + r0[q].y, x0[q][2] + r0[q].z, r0[q].w,
                     r1[q].x, r1[q].y);
        T.acc[l] = make_float4(0.f, 0.f, 0.f, __int_as_float(sl[q]));
      }
    }
  }
}

// The persistent task kernel.  Tasks are claimed from one counter in task order, one
// ahead of the running one.  Before task t runs, warp 0 moves t's descriptor (copied
// into shared memory while the previous task ran) into place, claims the next task and
// polls t's dependencies' progress counters -- one round trip for both when the
// dependencies are met -- and starts copying the next task's descriptor (cp.async),
// which lands while t runs; after t, a thread of the last warp publishes while warp 0
// already polls for the next task.  A task waits only for tasks earlier in the order,
// and the earliest unfinished claimed task is always some CTA's current one, so holding
// a claimed task cannot deadlock (only a running CTA claims, so this holds however many
// CTAs are resident; the grid is one round of them).  The
// loop keeps no counter: only shared memory carries state from one task to the next,
// which leaves the element loop all 80 registers.
template <int MODE, int BS>
__global__ void __launch_bounds__(BS, 768 / BS) k_flow_qp10(FlowArgs F, ElemParams ep,
                                                          NodeParams np) {
  extern __shared__ float sm[];
  __shared__ float red[BS / 32];
  __shared__ int sh_cur, sh_next, sh_ok;
  int* const dcur = reinterpret_cast<int*>(sm);      // the running task's descriptor
  int* const dnext = dcur + F.desc_stride;            // the next one's, arriving
  const bool w0 = threadIdx.x < 32;
  if (threadIdx.x == 0) sh_next = atomicAdd(F.task_ctr, 1);
  __syncthreads();
  if (w0 && sh_next < F.C + 2 * F.C * F.nsteps) flow_fetch(F, sh_next, dnext);
  for (;;) {
    if (w0) {
      const int ntasks = F.C + 2 * F.C * F.nsteps;
      const int t = sh_next;
      cp_async_wait();  // t's descriptor (copied by this warp)
      __syncwarp();
      for (int k = threadIdx.x; k < F.desc_stride; k += 32) dcur[k] = dnext[k];
      __syncwarp();
      bool ok = true;
      int tn = ntasks;
      if (t < ntasks) {
        int j, r;
        bool elem;
        flow_decode(t, F.C, j, r, elem);
        if (threadIdx.x == 0) tn = atomicAdd(F.task_ctr, 1);
        ok = elem ? flow_wait(F, F.node_done, dcur + kFlowDescHead, dcur[kFlowDescCount], j)
                  : (j == 0 || flow_wait(F, F.elem_done, dcur + kFlowDescHead,
                                         dcur[kFlowDescCount], j - 1));
        tn = __shfl_sync(0xffffffffu, tn, 0);
        if (ok && tn < ntasks) flow_fetch(F, tn, dnext);
      }
      if (threadIdx.x == 0) {
        sh_cur = t;
        sh_ok = ok;
        sh_next = tn;
      }
    }
    __syncthreads();
    const int t = sh_cur;
    if (t >= F.C + 2 * F.C * F.nsteps || !sh_ok) break;
    int j, r;
    bool elem;
    flow_decode(t, F.C, j, r, elem);
    // the descriptor is read here only: after the task's last barrier warp 0 overwrites
    // it with the next task's
    ChunkInfo ch;
    memcpy(&ch, dcur, sizeof(ChunkInfo));
    const int c = dcur[kFlowDescChunk];
    if (elem) {
      const Tile T = make_tile(sm + 2 * F.desc_stride, ch.n_local);
      flow_stage<BS>(F, ch, T, j);
      __syncthreads();
      float wint, wp;
      qp10_element_loop<MODE, BS, true, true>(F.A[0], ep, ch, T, threadIdx.x, wint, wp);
      __syncthreads();
      node_epilogue<BS>(F.A[j & 1], ch, T, threadIdx.x);
      if (ep.accum_energy) add_chunk_work<BS>(F.A[0], c, wint, wp, red);
      __syncthreads();
      if (threadIdx.x == BS - 32 && c != F.stall_chunk) flow_publish(F.elem_done, c, j);
    } else {
      flow_nodes<BS>(F, ep, np, ch, j);
      __syncthreads();
      if (threadIdx.x == BS - 32 && c != F.stall_chunk) flow_publish(F.node_done, c, j);
    }
  }
  if (w0) cp_async_wait();
}

// ---------------------------------------------------------------------------
// tet10, one thread per element, all four Gauss points, in barycentric form.
//
// With g_0 = e_xi, g_1 = e_eta, g_2 = -(1,1,1), g_3 = e_zeta the gradients of the
// barycentrics, corner k has grad N_k = (A_k - 1) g_k and edge (k,l) has
// grad N_kl = A_l g_k + A_k g_l (A = 4L).  At Gauss point p one barycentric is a and
// the other three b (corner kappa(p) = 2, 0, 1, 3 for p = 0..3), so A_m = 4b + 4(a-b)
// [m == kappa].  Hence
//   J_p = sum_k C_k g_k^T,  C_k = Y_k + 4(a-b) (k == kappa ? x_kappa : x_{k,kappa}),
//   Y_k = (4b-1) x_k + 4b sum_{l != k} x_{kl}       (the same at every point),
// and with Q_k(p) = P_p g_k (P = w detJ sigma J^-T) the element forces are
//   f_k  = (4b-1) S_k + 4(a-b) Q_k(p(k)),
//   f_kl = 4b (S_k + S_l) + 4(a-b) (Q_k(p(l)) + Q_l(p(k))),   S_k = sum_p Q_k(p),
// where p(k) is the point at which corner k carries the weight a.  Every index is
// known at compile time: about half the arithmetic of the per-node sums, no shuffles.
// ---------------------------------------------------------------------------
// edge node of corners k != l (CalculiX order 4:(0,1) 5:(1,2) 6:(2,0) 7:(0,3) 8:(1,3) 9:(2,3))
__device__ __host__ __forceinline__ constexpr int t10_edge(int k, int l) {
  const int lo = k < l ? k : l, hi = k < l ? l : k;
  return lo == 0 ? (hi == 1 ? 4 : hi == 2 ? 6 : 7) : lo == 1 ? (hi == 2 ? 5 : 8) : 9;
}
__device__ __host__ __forceinline__ constexpr int t10_kappa(int p) { return p == 0 ? 2 : p == 1 ? 0 : p == 2 ? 1 : 3; }

template <int MODE>
__device__ __forceinline__ void tet10_bary_element(const ElemParams& ep, const FusedArgs& A, int e,
                                                   const Tile& T, const int (&ln)[10],
                                                   float (&F)[10][3], float& wint, float& wp) {
  constexpr float qa = 0.58541019662496845f, qb = 0.13819660112501052f;
  constexpr float AL = 4.f * qb - 1.f, BE = 4.f * qb, GA = 4.f * (qa - qb);
  constexpr float W = 1.0f / 24.0f;
  // Y_k for positions (Yx) and increments (Yd), corners k = 0..3
  float Yx[4][3], Yd[4][3];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float2 pr[3];
    load_pairs(T, ln[k], pr);
    Yx[k][0] = AL * pr[0].x; Yx[k][1] = AL * pr[1].x; Yx[k][2] = AL * pr[2].x;
    Yd[k][0] = AL * pr[0].y; Yd[k][1] = AL * pr[1].y; Yd[k][2] = AL * pr[2].y;
  }
#pragma unroll
  for (int k = 0; k < 4; k++)
#pragma unroll
    for (int l = k + 1; l < 4; l++) {
      const int m = t10_edge(k, l);
      float2 pr[3];
      load_pairs(T, ln[m], pr);
      const float xs[3] = {pr[0].x, pr[1].x, pr[2].x}, ds[3] = {pr[0].y, pr[1].y, pr[2].y};
#pragma unroll
      for (int c = 0; c < 3; c++) {
        Yx[k][c] = fmaf(BE, xs[c], Yx[k][c]);
        Yx[l][c] = fmaf(BE, xs[c], Yx[l][c]);
        Yd[k][c] = fmaf(BE, ds[c], Yd[k][c]);
        Yd[l][c] = fmaf(BE, ds[c], Yd[l][c]);
      }
    }
  float Sq[3][3];  // S_k for k = 0, 1, 3 (rows), component c
#pragma unroll
  for (int i = 0; i < 3; i++) Sq[i][0] = Sq[i][1] = Sq[i][2] = 0.f;
#pragma unroll
  for (int i = 0; i < 10; i++) F[i][0] = F[i][1] = F[i][2] = 0.f;
#pragma unroll
  for (int p = 0; p < 4; p++) {
    const int kap = t10_kappa(p);
    // C_k = Y_k + GA * (point node of k at p)
    float Cx[4][3], Cd[4][3];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int m = k == kap ? k : t10_edge(k, kap);
      float2 pr[3];
      load_pairs(T, ln[m], pr);
      Cx[k][0] = fmaf(GA, pr[0].x, Yx[k][0]);
      Cx[k][1] = fmaf(GA, pr[1].x, Yx[k][1]);
      Cx[k][2] = fmaf(GA, pr[2].x, Yx[k][2]);
      Cd[k][0] = fmaf(GA, pr[0].y, Yd[k][0]);
      Cd[k][1] = fmaf(GA, pr[1].y, Yd[k][1]);
      Cd[k][2] = fmaf(GA, pr[2].y, Yd[k][2]);
    }
    float J[9], Gu[9];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      J[3 * a + 0] = Cx[0][a] - Cx[2][a];
      J[3 * a + 1] = Cx[1][a] - Cx[2][a];
      J[3 * a + 2] = Cx[3][a] - Cx[2][a];
      Gu[3 * a + 0] = Cd[0][a] - Cd[2][a];
      Gu[3 * a + 1] = Cd[1][a] - Cd[2][a];
      Gu[3 * a + 2] = Cd[3][a] - Cd[2][a];
    }
    float Ji[9];
    const float detJ = inv3f(J, Ji);
    if (!(detJ > 0.f)) atomicOr(A.status, (unsigned)ST_DEGENERATE);
    const float wd = W * detJ;
    float Lg[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++)
        Lg[3 * a + b] = Gu[3 * a + 0] * Ji[0 * 3 + b] + Gu[3 * a + 1] * Ji[1 * 3 + b] +
                        Gu[3 * a + 2] * Ji[2 * 3 + b];
    const float de[6] = {Lg[0], Lg[4], Lg[8], Lg[1] + Lg[3], Lg[5] + Lg[7], Lg[2] + Lg[6]};
    const float tr = de[0] + de[1] + de[2];
    float s[6];
    if (MODE == EM_REFCOMPAT) {
      s[0] = ep.lambda * tr + 2.f * ep.mu * de[0];
      s[1] = ep.lambda * tr + 2.f * ep.mu * de[1];
      s[2] = ep.lambda * tr + 2.f * ep.mu * de[2];
      s[3] = ep.mu * de[3];
      s[4] = ep.mu * de[4];
      s[5] = ep.mu * de[5];
      if (ep.accum_energy) {
        float w = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) w = fmaf(s[k], de[k], w);
        wint = fmaf(0.5f * wd, w, wint);
      }
    } else {
      const size_t qi = (size_t)e * 4 + p;
      const float4 sa = A.sig_a[qi];
      const float2 sb = A.sig_b[qi];
      const float ep0 = A.epbar[qi];
      const float s0[6] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y};
      s[0] = s0[0] + ep.lambda * tr + 2.f * ep.mu * de[0];
      s[1] = s0[1] + ep.lambda * tr + 2.f * ep.mu * de[1];
      s[2] = s0[2] + ep.lambda * tr + 2.f * ep.mu * de[2];
      s[3] = s0[3] + ep.mu * de[3];
      s[4] = s0[4] + ep.mu * de[4];
      s[5] = s0[5] + ep.mu * de[5];
      float epn = ep0;
      j2_return(ep, s, epn);
      A.sig_a[qi] = make_float4(s[0], s[1], s[2], s[3]);
      A.sig_b[qi] = make_float2(s[4], s[5]);
      A.epbar[qi] = epn;
      if (ep.accum_energy) {
        float w = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) w = fmaf(s0[k] + s[k], de[k], w);
        wint = fmaf(0.5f * wd, w, wint);
        wp = fmaf(wd * (ep.sy0 + ep.H * epn), epn - ep0, wp);
      }
    }
    const float Sg[9] = {s[0], s[3], s[5], s[3], s[1], s[4], s[5], s[4], s[2]};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float Pr[3];  // row c of P
#pragma unroll
      for (int j = 0; j < 3; j++)
        Pr[j] = wd * (Sg[3 * c + 0] * Ji[3 * j + 0] + Sg[3 * c + 1] * Ji[3 * j + 1] +
                      Sg[3 * c + 2] * Ji[3 * j + 2]);
      // Q_k = P g_k: Q_0 = P_0, Q_1 = P_1, Q_3 = P_2, Q_2 = -(P_0 + P_1 + P_2)
      const float Q[4] = {Pr[0], Pr[1], -(Pr[0] + Pr[1] + Pr[2]), Pr[2]};
      Sq[0][c] += Q[0];
      Sq[1][c] += Q[1];
      Sq[2][c] += Q[3];
      // the point terms of this point: corner kappa and the edges (kappa, l)
      F[kap][c] = fmaf(GA, Q[kap], F[kap][c]);
#pragma unroll
      for (int l = 0; l < 4; l++)
        if (l != kap) F[t10_edge(kap, l)][c] = fmaf(GA, Q[l], F[t10_edge(kap, l)][c]);
    }
  }
  // the smooth terms: corners (4b-1) S_k, edges 4b (S_k + S_l)
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float S[4] = {Sq[0][c], Sq[1][c], -(Sq[0][c] + Sq[1][c] + Sq[2][c]), Sq[2][c]};
#pragma unroll
    for (int k = 0; k < 4; k++) F[k][c] = fmaf(AL, S[k], F[k][c]);
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int l = k + 1; l < 4; l++)
        F[t10_edge(k, l)][c] = fmaf(BE, S[k] + S[l], F[t10_edge(k, l)][c]);
  }
}

// Fused tet10 step, one thread per element (tet10_bary_element).  4 CTAs of 128
// threads per SM (at most 128 registers).
template <int MODE, int BS, bool BATCH = false>
__global__ void __launch_bounds__(BS, 512 / BS) k_step_t10(FusedArgs A, ElemParams ep_arg, NodeParams np_arg) {
  extern __shared__ float sm[];
  const DevPlan& P = A.P;
  const ChunkInfo ch = P.chunks[blockIdx.x];
  const ChunkStep cs = chunk_step<BATCH>(A, ch, ep_arg, np_arg);
  if (cs.mode == 2) return;
  const ElemParams& ep = cs.ep;
  const Tile T = make_tile(sm, ch.n_local);
  __shared__ float red[BS / 32];

#ifndef CI_T10_STAGE_K
#define CI_T10_STAGE_K 4
#endif
  stage_nodes_k<BS, CI_T10_STAGE_K>(A, ep, cs.np, ch, cs.state_final, T, threadIdx.x);
  if (cs.mode == 1) return;
  __syncthreads();

  float wint = 0.f, wp = 0.f;
  const int E = P.E;
  for (int w = ch.elem_begin; w < ch.elem_end; w += BS) {
    const int e = w + threadIdx.x;
    const bool act = e < ch.elem_end;
    int col = -1;
    int ln[10];
    float f[10][3];
    if (act) {
      col = P.color[e];
#pragma unroll
      for (int a = 0; a < 10; a++) ln[a] = P.conn_local[(size_t)a * E + e];
      tet10_bary_element<MODE>(ep, A, e, T, ln, f, wint, wp);
    }
    const int c0 = P.color[w];
    const int c1 = P.color[min(w + BS, ch.elem_end) - 1];
    for (int k = c0; k <= c1; k++) {
      __syncthreads();
      if (col == k) {
#pragma unroll
        for (int a = 0; a < 10; a++) {
          float4 t = T.acc[ln[a]];
          t.x += f[a][0];
          t.y += f[a][1];
          t.z += f[a][2];
          T.acc[ln[a]] = t;
        }
      }
    }
  }
  __syncthreads();
  node_epilogue<BS>(A, ch, T, threadIdx.x);
  if (ep.accum_energy) add_chunk_work<BS>(A, blockIdx.x, wint, wp, red);
}

// S^N of every node after the last fused step of a call: reads S^{N-1} from the prv
// buffer and the halo of step N-1, writes S^N (and a^N) to the cur buffer.
static __global__ void __launch_bounds__(256) k_finalize_nodes(FusedArgs A, NodeParams np) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.P.N) return;
  double u[3], v[3];
  float a[3], uf[3], vf[3];
  bool hit;
  complete_node(A, np, g, A.P.slot_row[g], A.P.slot_row[g + 1], u, v, a, hit, uf, vf);
  store_node(A, A.u_cur, A.v_cur, g, u, v, vf, a, hit, A.store_acc != 0, A.contact[g]);
}

// a0 from zero internal force (wall at the start positions, gravity) and the half step
// v += dt/2 a0 (include/dynamics.h:454-463), rounded like node_step.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_node_init(NodeArrays A, NodeParams p_arg,
                                                   const NodeParams* inst_np, const int* node_inst,
                                                   const float* d0f) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= p_arg.N) return;
  const NodeParams p = BATCH ? inst_np[node_inst[n]] : p_arg;
  double u[3], v[3], ad[3];
  float uf[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    u[k] = A.u[k][n];
    v[k] = A.v[k][n];
    uf[k] = (float)u[k];
    ad[k] = (double)p.gf[k];
  }
  const float d32 = __fadd_rn(d0f[n], __fadd_rn(__fmul_rn(p.nf[0], uf[0]),
                                  __fadd_rn(__fmul_rn(p.nf[1], uf[1]), __fmul_rn(p.nf[2], uf[2]))));
  const float margin = 1e-6f * (1.f + fabsf(d0f[n]) + fabsf(uf[0]) + fabsf(uf[1]) + fabsf(uf[2]));
  unsigned char flag = 0;
  if (!(d32 > margin)) {
    const double d = __fma_rn(p.wall_n[2], u[2], __fma_rn(p.wall_n[1], u[1],
                              __fma_rn(p.wall_n[0], u[0], A.d0[n])));
    if (d < 0.0) {
      flag = 3;
      const double c = __ddiv_rn(__dmul_rn(-d, p.wall_k), (double)A.mass[n]);
#pragma unroll
      for (int k = 0; k < 3; k++) ad[k] = __fma_rn(c, p.wall_n[k], ad[k]);
    }
  }
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double vn = __fma_rn(0.5 * p.dt, ad[k], v[k]);
    finite = finite && isfinite((float)vn);
    A.v[k][n] = vn;
    A.acc[k][n] = (float)ad[k];
  }
  A.contact[n] = flag;
  if (!finite) atomicOr(A.status, (unsigned)ST_NONFINITE);
}

// Adds n to the batched step counter (after each captured block of steps).
static __global__ void k_tick(int* step_ctr, int n) { *step_ctr += n; }

// Peak |u| over a node range since the last reset (one FP32 max per block, fixed order).
static __global__ void k_peak_disp(const double* ux, const double* uy, const double* uz,
                                   const int* node_inst, float* inst_peak, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const float m = (float)sqrt(ux[n] * ux[n] + uy[n] * uy[n] + uz[n] * uz[n]);
  // non-negative floats order like their bit patterns: integer max is exact and
  // order-independent
  atomicMax(reinterpret_cast<int*>(inst_peak) + node_inst[n], __float_as_int(m));
}

// Lumped mass: sum of the node's slots (component 0) in chunk order.
static __global__ void k_mass_sum(const float* slot_m, const int* slot_row, float* mass, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float m = 0.f;
  for (int s = slot_row[n]; s < slot_row[n + 1]; s++) m += slot_m[s];
  mass[n] = m;
}

// Assembled internal force of a one-shot call: slot sums to FP64 [3][N].
static __global__ void k_force_sum(const float* sx, const float* sy, const float* sz, const int* slot_row,
                            double* f, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float a = 0.f, b = 0.f, c = 0.f;
  for (int s = slot_row[n]; s < slot_row[n + 1]; s++) {
    a += sx[s];
    b += sy[s];
    c += sz[s];
  }
  f[n] = a;
  f[N + n] = b;
  f[2 * (size_t)N + n] = c;
}

// Energy terms at the current state, one FP64 partial per block (fixed-order sums):
// out[blk][0] kinetic (v_n = v - dt/2 a), [1] contact potential, [2] gravity work.
static __global__ void k_energy(NodeArrays A, NodeParams p, double* out) {
  __shared__ double red[3][256];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0, phi = 0.0, wg = 0.0;
  if (n < p.N) {
    const double m = A.mass[n];
    double v2 = 0.0;
    for (int k = 0; k < 3; k++) {
      const double vn = A.v[k][n] - 0.5 * p.dt * (double)A.acc[k][n];
      v2 += vn * vn;
      wg += m * p.g[k] * A.u[k][n];
    }
    ke = 0.5 * m * v2;
    const double d = A.d0[n] + p.wall_n[0] * A.u[0][n] + p.wall_n[1] * A.u[1][n] +
                     p.wall_n[2] * A.u[2][n];
    if (d < 0.0) phi = 0.5 * p.wall_k * d * d;
  }
  red[0][threadIdx.x] = ke;
  red[1][threadIdx.x] = phi;
  red[2][threadIdx.x] = wg;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; k++) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; k++) out[3 * (size_t)blockIdx.x + k] = red[k][0];
}

}  // namespace ci
