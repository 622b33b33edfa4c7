// solver64.cpp -- TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// FP64 restatement of the GB300 solver's formulation.  The CUDA kernels compute the
// same quantities in FP32 (element math) with FP64 nodal state; this file is the
// "FP64 run of the same solver" that their results are measured against.
//
// Formulation (per step n, state x^n, v^{n+1/2}):
//   du      = dt v^{n+1/2}                                   (include/dynamics.h:477-479)
//   per QP: J = sum_i x_i (x) dN_i/dxi at x^n, dN/dx = J^-T dN/dxi,
//           d_eps = sym(grad du)                              (B du, include/analysis.h:321-382)
//           RefCompat: sigma = D d_eps  (no stored stress: f = K_e(x^n) du)
//           J2:        sigma = radial_return(sigma_n + D d_eps)
//           f_i += w detJ sigma . dN_i/dx
//   a  = -f/m + wall(x^n + du) + g                             (include/dynamics_kernels.h:150-168)
//   x^{n+1} = x^n + du ; v^{n+3/2} = v^{n+1/2} + dt a         (include/dynamics.h:497-503)
// Quadrature: 1 point for tet4 (B is constant, so K_e equals the reference's 5-point
// K_e up to its truncated weights), 4-point Gauss for tet10 (degree 2, exact for the
// straight-sided K_e and row-sum mass).
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

const double kAlpha = 0.58541019662496845446;  // (5 + 3 sqrt5) / 20
const double kBeta = 0.13819660112501051518;   // (5 - sqrt5) / 20

struct Rule {
  int nq;
  double pt[4][3];
  double w[4];
};

Rule rule_for(int npe) {
  Rule r;
  if (npe == 4) {
    r.nq = 1;
    r.pt[0][0] = r.pt[0][1] = r.pt[0][2] = 0.25;
    r.w[0] = 1.0 / 6.0;
  } else {
    r.nq = 4;
    const double P[4][3] = {{kBeta, kBeta, kBeta}, {kAlpha, kBeta, kBeta}, {kBeta, kAlpha, kBeta},
                            {kBeta, kBeta, kAlpha}};
    std::memcpy(r.pt, P, sizeof(P));
    for (int q = 0; q < 4; q++) r.w[q] = 1.0 / 24.0;
  }
  return r;
}

// Barycentrics of the reference's element parametrisation:
// node 0 <-> xi, node 1 <-> eta, node 2 <-> 1-xi-eta-zeta, node 3 <-> zeta
// (include/tetrahedral.h:182-197, 521-531).
void shape(int npe, const double* p, double* N) {
  if (npe == 4) {
    N[0] = 1.0 - p[0] - p[1] - p[2];
    N[1] = p[0];
    N[2] = p[1];
    N[3] = p[2];
    return;
  }
  const double L[4] = {p[0], p[1], 1.0 - p[0] - p[1] - p[2], p[2]};
  static const int ed[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  for (int c = 0; c < 4; c++) N[c] = L[c] * (2.0 * L[c] - 1.0);
  for (int k = 0; k < 6; k++) N[4 + k] = 4.0 * L[ed[k][0]] * L[ed[k][1]];
}

void shape_grad(int npe, const double* p, double* G) {
  if (npe == 4) {
    const double g[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::memcpy(G, g, sizeof(g));
    return;
  }
  const double L[4] = {p[0], p[1], 1.0 - p[0] - p[1] - p[2], p[2]};
  const double dL[4][3] = {{1, 0, 0}, {0, 1, 0}, {-1, -1, -1}, {0, 0, 1}};
  static const int ed[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  for (int c = 0; c < 4; c++)
    for (int j = 0; j < 3; j++) G[3 * c + j] = (4.0 * L[c] - 1.0) * dL[c][j];
  for (int k = 0; k < 6; k++) {
    const int a = ed[k][0], b = ed[k][1];
    for (int j = 0; j < 3; j++) G[3 * (4 + k) + j] = 4.0 * (L[a] * dL[b][j] + L[b] * dL[a][j]);
  }
}

double inv3(const double* A, double* Ai) {
  const double c00 = A[4] * A[8] - A[5] * A[7];
  const double c01 = A[5] * A[6] - A[3] * A[8];
  const double c02 = A[3] * A[7] - A[4] * A[6];
  const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  const double r = 1.0 / det;
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

// Per QP: dN/dx [npe][3] and detJ from element coordinates xe [npe][3].
double qp_geometry(int npe, const double* pt, const double* xe, double* dNdx) {
  double G[30], J[9], Ji[9];
  shape_grad(npe, pt, G);
  for (int a = 0; a < 9; a++) J[a] = 0.0;
  for (int i = 0; i < npe; i++)
    for (int p = 0; p < 3; p++)
      for (int q = 0; q < 3; q++) J[3 * p + q] += xe[3 * i + p] * G[3 * i + q];
  const double detJ = inv3(J, Ji);
  for (int i = 0; i < npe; i++)
    for (int c = 0; c < 3; c++)
      dNdx[3 * i + c] = Ji[0 * 3 + c] * G[3 * i + 0] + Ji[1 * 3 + c] * G[3 * i + 1] +
                        Ji[2 * 3 + c] * G[3 * i + 2];
  return detJ;
}

struct Elastic {
  double mu, lambda;
};

Elastic lame(double E, double nu) {
  Elastic e;
  e.mu = E / (2.0 * (1.0 + nu));
  e.lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  return e;
}

void j2_update(const Elastic& el, double sy0, double H, const double* de, double* s,
               double* epbar, bool plastic) {
  const double tr = de[0] + de[1] + de[2];
  double t[6];
  for (int k = 0; k < 3; k++) t[k] = s[k] + el.lambda * tr + 2.0 * el.mu * de[k];
  for (int k = 3; k < 6; k++) t[k] = s[k] + el.mu * de[k];
  if (plastic) {
    const double p = (t[0] + t[1] + t[2]) / 3.0;
    double d[6] = {t[0] - p, t[1] - p, t[2] - p, t[3], t[4], t[5]};
    const double nrm = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] +
                                 2.0 * (d[3] * d[3] + d[4] * d[4] + d[5] * d[5]));
    const double f = nrm - std::sqrt(2.0 / 3.0) * (sy0 + H * (*epbar));
    if (f > 0.0) {
      const double dg = f / (2.0 * el.mu + 2.0 * H / 3.0);
      const double scale = 1.0 - 2.0 * el.mu * dg / nrm;
      for (int k = 0; k < 6; k++) d[k] *= scale;
      t[0] = d[0] + p;
      t[1] = d[1] + p;
      t[2] = d[2] + p;
      t[3] = d[3];
      t[4] = d[4];
      t[5] = d[5];
      *epbar += std::sqrt(2.0 / 3.0) * dg;
    }
  }
  std::memcpy(s, t, sizeof(t));
}

void gather3(int npe, const int* nodes, const double* src, double* dst) {
  for (int j = 0; j < npe; j++)
    for (int k = 0; k < 3; k++) dst[3 * j + k] = src[3 * (size_t)nodes[j] + k];
}

}  // namespace

extern "C" int orc_num_qp(int npe) { return npe == 4 ? 1 : (npe == 10 ? 4 : 0); }

extern "C" void orc_j2_update(double E, double nu, double sigma_y0, double H,
                              const double d_eps[6], double sigma[6], double* epbar) {
  j2_update(lame(E, nu), sigma_y0, H, d_eps, sigma, epbar, true);
}

extern "C" int orc_lumped_mass(const orc_mesh* m, const orc_params* p, const double* xloc,
                               double* mass) {
  const int npe = m->nodes_per_element;
  if (npe != 4 && npe != 10) return -1;
  const Rule r = rule_for(npe);
  std::memset(mass, 0, sizeof(double) * m->num_nodes);
  double xe[30], dNdx[30], N[10];
  for (int e = 0; e < m->num_elements; e++) {
    const int* nodes = m->conn + (size_t)npe * e;
    gather3(npe, nodes, xloc, xe);
    double me[10] = {0}, vol = 0.0;
    for (int q = 0; q < r.nq; q++) {
      const double wd = r.w[q] * qp_geometry(npe, r.pt[q], xe, dNdx);
      vol += wd;
      shape(npe, r.pt[q], N);
      for (int i = 0; i < npe; i++) me[i] += p->rho * N[i] * wd;
    }
    if (p->lumping == ORC_LUMP_HRZ && npe == 10) {
      // HRZ: diagonal of the consistent mass scaled to the element mass.  For the
      // straight-sided tet10, M_ii = rho V {6,6,6,6,32,...}/420, so the lumped
      // masses are rho V / 36 (corners) and 4 rho V / 27 (edges).
      for (int i = 0; i < 4; i++) me[i] = p->rho * vol / 36.0;
      for (int i = 4; i < 10; i++) me[i] = 4.0 * p->rho * vol / 27.0;
    }
    for (int i = 0; i < npe; i++) mass[nodes[i]] += me[i];
  }
  return 0;
}

namespace {

// One element's internal force fe[3 npe] at positions x with increment du, its QP
// states updated in place (sigma/epbar may be NULL: zero stored state, not written),
// and its internal-work and plastic-dissipation increments added to *wint / *wp in
// QP order.
void element_force(int npe, const Rule& r, const Elastic& el, const orc_params* p, bool j2,
                   const int* nodes, const double* x, const double* du, const double* sigma_in,
                   const double* epbar_in, double* sigma_out, double* epbar_out, size_t e,
                   double* fe, double* wint, double* wp) {
  double xe[30], de[30], dNdx[30];
  gather3(npe, nodes, x, xe);
  gather3(npe, nodes, du, de);
  for (int i = 0; i < 3 * npe; i++) fe[i] = 0.0;
  for (int q = 0; q < r.nq; q++) {
    const double detJ = qp_geometry(npe, r.pt[q], xe, dNdx);
    const double wd = r.w[q] * detJ;
    double L[9] = {0};
    for (int i = 0; i < npe; i++)
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) L[3 * a + b] += de[3 * i + a] * dNdx[3 * i + b];
    const double deps[6] = {L[0], L[4], L[8], L[1] + L[3], L[5] + L[7], L[2] + L[6]};
    const size_t qi = e * r.nq + q;
    double s[6] = {0, 0, 0, 0, 0, 0}, s0[6] = {0, 0, 0, 0, 0, 0}, ep = 0.0;
    if (j2 && sigma_in) std::memcpy(s, sigma_in + 6 * qi, sizeof(s));
    if (j2 && epbar_in) ep = epbar_in[qi];
    std::memcpy(s0, s, sizeof(s));
    const double ep0 = ep;
    j2_update(el, p->sigma_y0, p->H, deps, s, &ep, j2);
    if (sigma_out) std::memcpy(sigma_out + 6 * qi, s, sizeof(s));
    if (epbar_out) epbar_out[qi] = ep;
    double wq = 0.0;
    for (int k = 0; k < 6; k++) wq += 0.5 * (s0[k] + s[k]) * deps[k];
    *wint += wd * wq;
    *wp += wd * (p->sigma_y0 + p->H * ep) * (ep - ep0);
    const double S[9] = {s[0], s[3], s[5], s[3], s[1], s[4], s[5], s[4], s[2]};
    for (int i = 0; i < npe; i++)
      for (int a = 0; a < 3; a++)
        fe[3 * i + a] += wd * (S[3 * a + 0] * dNdx[3 * i + 0] + S[3 * a + 1] * dNdx[3 * i + 1] +
                               S[3 * a + 2] * dNdx[3 * i + 2]);
  }
}

// Fork-join pool for the solver's loops: run(fn) calls fn(t) on threads t = 0..n-1
// (t = 0 on the caller) and returns when all are done.
class Pool {
 public:
  explicit Pool(int n) : n_(n < 1 ? 1 : n) {
    for (int t = 1; t < n_; t++) th_.emplace_back([this, t] { worker(t); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
      gen_++;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  int size() const { return n_; }
  void run(const std::function<void(int)>& fn) {
    if (n_ == 1) {
      fn(0);
      return;
    }
    {
      std::lock_guard<std::mutex> l(mu_);
      fn_ = &fn;
      pending_ = n_ - 1;
      gen_++;
    }
    cv_.notify_all();
    fn(0);
    std::unique_lock<std::mutex> l(mu_);
    done_.wait(l, [this] { return pending_ == 0; });
  }

 private:
  void worker(int t) {
    unsigned long long seen = 0;
    for (;;) {
      const std::function<void(int)>* fn;
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        fn = fn_;
      }
      (*fn)(t);
      std::lock_guard<std::mutex> l(mu_);
      if (--pending_ == 0) done_.notify_one();
    }
  }
  int n_;
  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* fn_ = nullptr;
  int pending_ = 0;
  unsigned long long gen_ = 0;
  bool stop_ = false;
};

// contiguous share [b, e) of n items for thread t of T
inline void share(size_t n, int t, int T, size_t* b, size_t* e) {
  *b = n * (size_t)t / (size_t)T;
  *e = n * (size_t)(t + 1) / (size_t)T;
}

constexpr size_t kBlock = 1024;  // elements per work-sum block (fixed: thread-count independent)

}  // namespace

extern "C" int orc_internal_force(const orc_mesh* m, const orc_params* p, const double* x,
                                  const double* du, const double* sigma_in,
                                  const double* epbar_in, double* f, double* sigma_out,
                                  double* epbar_out, double* work) {
  const int npe = m->nodes_per_element;
  if (npe != 4 && npe != 10) return -1;
  const Rule r = rule_for(npe);
  const Elastic el = lame(p->E, p->nu);
  const bool j2 = p->mode == ORC_J2;
  std::memset(f, 0, sizeof(double) * 3 * m->num_nodes);
  double Wint = 0.0, Wp = 0.0;
  double fe[30];
  for (int e = 0; e < m->num_elements; e++) {
    const int* nodes = m->conn + (size_t)npe * e;
    element_force(npe, r, el, p, j2, nodes, x, du, sigma_in, epbar_in, sigma_out, epbar_out,
                  (size_t)e, fe, &Wint, &Wp);
    for (int i = 0; i < npe; i++)
      for (int a = 0; a < 3; a++) f[3 * (size_t)nodes[i] + a] += fe[3 * i + a];
  }
  if (work) {
    work[0] = Wint;
    work[1] = Wp;
  }
  return 0;
}

struct orc_solver {
  orc_mesh m;
  orc_params p;
  int nq;
  std::vector<int> conn;
  std::vector<double> X0, X, x, v, a, mass, sigma, epbar, f, du, pos;
  std::vector<unsigned char> contact;
  double dt = 0.0, Wint = 0.0, Wp = 0.0, KE0 = 0.0, Phi0 = 0.0;
  // threaded step: per-element forces, per-block work sums, node -> (element, local
  // node) incidence in element order (so every node's force is summed in the order
  // of the one-thread loop)
  std::unique_ptr<Pool> pool;
  std::vector<double> fe_all, block_work;
  std::vector<long long> inc_row;
  std::vector<int> inc;
};

namespace {

// Wall and gravity on the accelerations of nodes [i0, i1); contact potential 1/2 k d^2
// of the penetration at p = x + du (planar generalisation of include/wall.h:37-43).
double apply_wall(orc_solver* s, const double* pos, double* acc, bool flag, size_t i0,
                  size_t i1) {
  const orc_params& P = s->p;
  double phi = 0.0;
  for (size_t i = i0; i < i1; i++) {
    const double* q = pos + 3 * i;
    const double d = P.wall_normal[0] * q[0] + P.wall_normal[1] * q[1] + P.wall_normal[2] * q[2] -
                     P.wall_offset;
    if (flag) s->contact[i] &= 2;
    if (d < 0.0) {
      const double c = -d * P.wall_stiffness / s->mass[i];
      for (int k = 0; k < 3; k++) acc[3 * i + k] += c * P.wall_normal[k];
      phi += 0.5 * P.wall_stiffness * d * d;
      if (flag) s->contact[i] |= 3;
    }
    for (int k = 0; k < 3; k++) acc[3 * i + k] += P.gravity[k];
  }
  return phi;
}

double contact_potential(const orc_solver* s, const double* pos) {
  double phi = 0.0;
  for (int i = 0; i < s->m.num_nodes; i++) {
    const double* q = pos + 3 * (size_t)i;
    const double d = s->p.wall_normal[0] * q[0] + s->p.wall_normal[1] * q[1] +
                     s->p.wall_normal[2] * q[2] - s->p.wall_offset;
    if (d < 0.0) phi += 0.5 * s->p.wall_stiffness * d * d;
  }
  return phi;
}

void build_incidence(orc_solver* s) {
  const size_t N = s->m.num_nodes, E = s->m.num_elements, npe = s->m.nodes_per_element;
  s->inc_row.assign(N + 1, 0);
  for (size_t k = 0; k < E * npe; k++) s->inc_row[s->conn[k] + 1]++;
  for (size_t i = 0; i < N; i++) s->inc_row[i + 1] += s->inc_row[i];
  s->inc.resize(E * npe);
  std::vector<long long> fill(s->inc_row.begin(), s->inc_row.end() - 1);
  for (size_t k = 0; k < E * npe; k++) s->inc[fill[s->conn[k]]++] = (int)k;  // element order
}

}  // namespace

extern "C" orc_solver* orc_create(const orc_mesh* m, const orc_params* p) {
  if (m->nodes_per_element != 4 && m->nodes_per_element != 10) return nullptr;
  orc_solver* s = new orc_solver();
  s->p = *p;
  s->nq = orc_num_qp(m->nodes_per_element);
  const size_t N = m->num_nodes, E = m->num_elements, npe = m->nodes_per_element;
  s->conn.assign(m->conn, m->conn + npe * E);
  s->X0.assign(m->xloc, m->xloc + 3 * N);
  s->m = *m;
  s->m.conn = s->conn.data();
  s->m.xloc = s->X0.data();
  s->X = s->x = s->X0;
  s->v.assign(3 * N, 0.0);
  s->a.assign(3 * N, 0.0);
  s->f.assign(3 * N, 0.0);
  s->du.assign(3 * N, 0.0);
  s->pos.assign(3 * N, 0.0);
  s->mass.assign(N, 0.0);
  s->sigma.assign(6 * E * s->nq, 0.0);
  s->epbar.assign(E * s->nq, 0.0);
  s->contact.assign(N, 0);
  s->pool.reset(new Pool(1));
  return s;
}

extern "C" void orc_destroy(orc_solver* s) { delete s; }

extern "C" int orc_set_threads(orc_solver* s, int nthreads) {
  if (nthreads < 1) return -1;
  s->pool.reset(new Pool(nthreads));
  return 0;
}

extern "C" int orc_initialize(orc_solver* s, const double pos[3], const double vel[3], double dt) {
  const int N = s->m.num_nodes;
  s->dt = dt;
  for (int i = 0; i < N; i++)
    for (int k = 0; k < 3; k++) {
      s->X[3 * i + k] = s->X0[3 * i + k] + pos[k];
      s->v[3 * i + k] = vel[k];
    }
  s->x = s->X;
  std::fill(s->sigma.begin(), s->sigma.end(), 0.0);
  std::fill(s->epbar.begin(), s->epbar.end(), 0.0);
  std::fill(s->contact.begin(), s->contact.end(), 0);
  s->Wint = s->Wp = 0.0;
  orc_lumped_mass(&s->m, &s->p, s->x.data(), s->mass.data());
  s->KE0 = 0.0;
  for (int i = 0; i < N; i++)
    s->KE0 += 0.5 * s->mass[i] * (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
  // a0 from a zero increment: f_int = 0 for zero stored stress (include/dynamics.h:454-463)
  std::fill(s->a.begin(), s->a.end(), 0.0);
  s->Phi0 = apply_wall(s, s->x.data(), s->a.data(), true, 0, (size_t)N);
  for (int i = 0; i < 3 * N; i++) s->v[i] += 0.5 * dt * s->a[i];
  return 0;
}

// One step per iteration: du = dt v; element forces (J2 update) in parallel over
// elements; each node's force summed over its elements in element order; a = -f/m +
// wall + gravity at x + du; x += du; v += dt a.  The result does not depend on the
// thread count: forces are summed per node in the one-thread loop's order and the
// work terms over fixed blocks of kBlock elements, in block order.
extern "C" int orc_step(orc_solver* s, int nsteps) {
  const size_t N = s->m.num_nodes, E = s->m.num_elements;
  const int npe = s->m.nodes_per_element;
  const double dt = s->dt;
  const Rule r = rule_for(npe);
  const Elastic el = lame(s->p.E, s->p.nu);
  const bool j2 = s->p.mode == ORC_J2;
  const size_t nblocks = (E + kBlock - 1) / kBlock;
  if (s->inc.empty()) build_incidence(s);
  s->fe_all.resize(E * 3 * npe);
  s->block_work.resize(2 * nblocks);
  Pool& pool = *s->pool;
  const int T = pool.size();
  for (int it = 0; it < nsteps; it++) {
    pool.run([&](int t) {
      size_t b, e;
      share(3 * N, t, T, &b, &e);
      for (size_t i = b; i < e; i++) s->du[i] = dt * s->v[i];
    });
    pool.run([&](int t) {
      for (size_t blk = t; blk < nblocks; blk += T) {
        double wi = 0.0, wpl = 0.0;
        const size_t e1 = std::min(E, (blk + 1) * kBlock);
        for (size_t e = blk * kBlock; e < e1; e++)
          element_force(npe, r, el, &s->p, j2, s->conn.data() + (size_t)npe * e, s->x.data(),
                        s->du.data(), j2 ? s->sigma.data() : nullptr,
                        j2 ? s->epbar.data() : nullptr, j2 ? s->sigma.data() : nullptr,
                        j2 ? s->epbar.data() : nullptr, e, s->fe_all.data() + 3 * npe * e, &wi,
                        &wpl);
        s->block_work[2 * blk] = wi;
        s->block_work[2 * blk + 1] = wpl;
      }
    });
    pool.run([&](int t) {
      size_t b, e;
      share(N, t, T, &b, &e);
      for (size_t i = b; i < e; i++) {
        double f[3] = {0.0, 0.0, 0.0};
        for (long long k = s->inc_row[i]; k < s->inc_row[i + 1]; k++) {
          const double* fe = s->fe_all.data() + 3 * (size_t)s->inc[k];
          for (int c = 0; c < 3; c++) f[c] += fe[c];
        }
        for (int c = 0; c < 3; c++) {
          s->a[3 * i + c] = -f[c] / s->mass[i];
          s->pos[3 * i + c] = s->x[3 * i + c] + s->du[3 * i + c];
        }
      }
      apply_wall(s, s->pos.data(), s->a.data(), true, b, e);
      for (size_t i = 3 * b; i < 3 * e; i++) {
        s->x[i] = s->pos[i];
        s->v[i] += dt * s->a[i];
      }
    });
    for (size_t blk = 0; blk < nblocks; blk++) {
      s->Wint += s->block_work[2 * blk];
      s->Wp += s->block_work[2 * blk + 1];
    }
  }
  return 0;
}

extern "C" int orc_get(const orc_solver* s, double* x, double* v, double* mass, double* sigma,
                       double* epbar, double* energy, unsigned char* contact) {
  const size_t N = s->m.num_nodes, E = s->m.num_elements;
  if (x) std::memcpy(x, s->x.data(), sizeof(double) * 3 * N);
  if (v) std::memcpy(v, s->v.data(), sizeof(double) * 3 * N);
  if (mass) std::memcpy(mass, s->mass.data(), sizeof(double) * N);
  if (sigma) std::memcpy(sigma, s->sigma.data(), sizeof(double) * 6 * E * s->nq);
  if (epbar) std::memcpy(epbar, s->epbar.data(), sizeof(double) * E * s->nq);
  if (contact) std::memcpy(contact, s->contact.data(), N);
  if (energy) {
    for (int k = 0; k < ORC_E_COUNT; k++) energy[k] = 0.0;
    double ke = 0.0, wg = 0.0;
    for (size_t i = 0; i < N; i++) {
      double v2 = 0.0;
      for (int k = 0; k < 3; k++) {
        const double vn = s->v[3 * i + k] - 0.5 * s->dt * s->a[3 * i + k];
        v2 += vn * vn;
        wg += s->mass[i] * s->p.gravity[k] * (s->x[3 * i + k] - s->X[3 * i + k]);
      }
      ke += 0.5 * s->mass[i] * v2;
    }
    const double phi = contact_potential(s, s->x.data());
    energy[ORC_E_KINETIC] = ke;
    energy[ORC_E_INTERNAL] = s->Wint;
    energy[ORC_E_PLASTIC] = s->Wp;
    energy[ORC_E_CONTACT] = -(phi - s->Phi0);
    energy[ORC_E_GRAVITY] = wg;
    energy[ORC_E_KINETIC0] = s->KE0;
    energy[ORC_E_BALANCE] = ke + s->Wint - energy[ORC_E_CONTACT] - wg - s->KE0;
  }
  return 0;
}
