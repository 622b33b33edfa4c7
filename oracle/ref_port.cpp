// ref_port.cpp -- TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// FP64 restatement of smdogroup/cppimpact's CPU path for the explicit impact step.
// Every function names the reference lines it follows.  The formulas, the truncated
// quadrature constants and the accumulation order are kept as the reference has
// them, because this file is the parity anchor: it must reproduce the reference's
// numbers to round-off (checked against the compiled reference through
// tests/golden/).  The one structural addition is an optional split of the element
// loop across threads for the timed CPU baseline.
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

// TetrahedralQuadrature5pts::get_quadrature_pt (include/tetrahedral.h:11-40).  The
// constants are truncated in the reference (weights sum to 0.16666666667, not 1/6);
// they are reproduced as written so that this port matches it to round-off.
const double kQ5Pt[5][3] = {{0.25, 0.25, 0.25},
                            {0.16666666666, 0.16666666666, 0.16666666666},
                            {0.5, 0.16666666666, 0.16666666666},
                            {0.16666666666, 0.5, 0.16666666666},
                            {0.16666666666, 0.16666666666, 0.5}};
const double kQ5W[5] = {-0.13333333333, 0.075, 0.075, 0.075, 0.075};

// Shape functions.  Linear: include/tetrahedral.h:521-549.  Quadratic (node order
// corners xi, eta, 1-xi-eta-zeta, zeta then edges): include/tetrahedral.h:182-250.
void shape(int npe, const double* p, double* N) {
  if (npe == 4) {
    N[0] = 1.0 - p[0] - p[1] - p[2];
    N[1] = p[0];
    N[2] = p[1];
    N[3] = p[2];
    return;
  }
  const double L1 = 1.0 - p[0] - p[1] - p[2], L2 = p[0], L3 = p[1], L4 = p[2];
  N[0] = (2 * L2 - 1) * L2;
  N[1] = (2 * L3 - 1) * L3;
  N[2] = (2 * L1 - 1) * L1;
  N[3] = (2 * L4 - 1) * L4;
  N[4] = 4 * L2 * L3;
  N[5] = 4 * L1 * L3;
  N[6] = 4 * L1 * L2;
  N[7] = 4 * L2 * L4;
  N[8] = 4 * L3 * L4;
  N[9] = 4 * L1 * L4;
}

// dN/dxi as [node][3].  The term order of each quadratic entry follows the
// reference expressions so that the rounding is the same.
void shape_grad(int npe, const double* p, double* G) {
  if (npe == 4) {
    const double g[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::memcpy(G, g, sizeof(g));
    return;
  }
  G[0] = 4 * p[0] - 1;  G[1] = 0.0;  G[2] = 0.0;
  G[3] = 0.0;  G[4] = 4 * p[1] - 1;  G[5] = 0.0;
  G[6] = 4 * p[0] + 4 * p[1] + 4 * p[2] - 3;
  G[7] = 4 * p[1] + 4 * p[0] + 4 * p[2] - 3;
  G[8] = 4 * p[2] + 4 * p[0] + 4 * p[1] - 3;
  G[9] = 0.0;  G[10] = 0.0;  G[11] = 4.0 * p[2] - 1.0;
  G[12] = 4 * p[1];  G[13] = 4 * p[0];  G[14] = 0.0;
  G[15] = -4 * p[1];  G[16] = -8 * p[1] - 4 * p[0] - 4 * p[2] + 4;  G[17] = -4 * p[1];
  G[18] = -8 * p[0] - 4 * p[1] - 4 * p[2] + 4;  G[19] = -4 * p[0];  G[20] = -4 * p[0];
  G[21] = 4 * p[2];  G[22] = 0.0;  G[23] = 4 * p[0];
  G[24] = 0.0;  G[25] = 4 * p[2];  G[26] = 4 * p[1];
  G[27] = -4 * p[2];  G[28] = -4 * p[2];  G[29] = -8 * p[2] - 4 * p[0] - 4 * p[1] + 4;
}

// Partition-of-unity gradients of the quadratic element
// (include/tetrahedral.h:289-340).  Only calculate_strain_energy observes them:
// there the inverse of the PU Jacobian overwrites Jinv (include/analysis.h:412-418).
void shape_grad_pu(const double* p, double* G) {
  G[0] = 2 * p[0];  G[1] = 0.0;  G[2] = 0.0;
  G[3] = 0.0;  G[4] = 2 * p[1];  G[5] = 0.0;
  G[6] = 2 * p[0] + 2 * p[1] + 2 * p[2] - 2;
  G[7] = 2 * p[1] + 2 * p[0] + 2 * p[2] - 2;
  G[8] = 2 * p[2] + 2 * p[0] + 2 * p[1] - 2;
  G[9] = 0.0;  G[10] = 0.0;  G[11] = 2 * p[2];
  G[12] = 2 * p[1];  G[13] = 2 * p[0];  G[14] = 0;
  G[15] = -2 * p[1];  G[16] = -4.0 * p[1] - 2.0 * p[0] - 2.0 * p[2] + 2.0;  G[17] = -2 * p[1];
  G[18] = -4.0 * p[0] - 2 * p[1] - 2 * p[2] + 2;  G[19] = -2 * p[0];  G[20] = -2 * p[0];
  G[21] = 2 * p[2];  G[22] = 0;  G[23] = 2 * p[0];
  G[24] = 0.0;  G[25] = 2 * p[2];  G[26] = 2 * p[1];
  G[27] = -2 * p[2];  G[28] = -2 * p[2];  G[29] = -4.0 * p[2] - 2.0 * p[0] - 2.0 * p[1] + 2.0;
}

// J[p][q] = sum_i dN_i/dxi_q x_{i,p}  (eval_grad, include/tetrahedral.h:252-269, 551-567)
void jacobian(int npe, const double* G, const double* x, double* J) {
  for (int a = 0; a < 9; a++) J[a] = 0.0;
  for (int p = 0; p < 3; p++)
    for (int q = 0; q < 3; q++)
      for (int i = 0; i < npe; i++) J[3 * p + q] += G[3 * i + q] * x[3 * i + p];
}

// inv3x3 (include/physics.h:38-58): cofactor inverse, returns the determinant.
double inverse3(const double* A, double* Ai) {
  const double det = (A[8] * (A[0] * A[4] - A[3] * A[1]) - A[7] * (A[0] * A[5] - A[3] * A[2]) +
                      A[6] * (A[1] * A[5] - A[2] * A[4]));
  const double r = 1.0 / det;
  Ai[0] = (A[4] * A[8] - A[5] * A[7]) * r;
  Ai[1] = -(A[1] * A[8] - A[2] * A[7]) * r;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * r;
  Ai[3] = -(A[3] * A[8] - A[5] * A[6]) * r;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * r;
  Ai[5] = -(A[0] * A[5] - A[2] * A[3]) * r;
  Ai[6] = (A[3] * A[7] - A[4] * A[6]) * r;
  Ai[7] = -(A[0] * A[7] - A[1] * A[6]) * r;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * r;
  return det;
}

// Strain-displacement matrix, 6 x 3npe, rows xx yy zz gxy gyz gxz
// (calculate_B_matrix, include/tetrahedral.h:442-484, 597-637).
void bmatrix(int npe, const double* Ji, const double* G, double* B) {
  const int n = 3 * npe;
  std::memset(B, 0, sizeof(double) * 6 * n);
  for (int a = 0; a < npe; a++) {
    double d[3];
    for (int i = 0; i < 3; i++) {
      d[i] = 0.0;
      for (int j = 0; j < 3; j++) d[i] += Ji[3 * j + i] * G[3 * a + j];
    }
    const int c = 3 * a;
    B[0 * n + c + 0] = d[0];
    B[1 * n + c + 1] = d[1];
    B[2 * n + c + 2] = d[2];
    B[3 * n + c + 0] = d[1];
    B[3 * n + c + 1] = d[0];
    B[4 * n + c + 1] = d[2];
    B[4 * n + c + 2] = d[1];
    B[5 * n + c + 0] = d[2];
    B[5 * n + c + 2] = d[0];
  }
}

// Isotropic elasticity matrix (calculate_D_matrix, include/tetrahedral.h:486-512).
void dmatrix(double E, double nu, double* D) {
  std::memset(D, 0, sizeof(double) * 36);
  D[0] = D[7] = D[14] = 1 - nu;
  D[21] = D[28] = D[35] = (1 - 2 * nu) / 2;
  D[1] = D[6] = nu;
  D[2] = D[12] = nu;
  D[8] = D[13] = nu;
  for (int i = 0; i < 36; i++) D[i] *= E / ((1 + nu) * (1 - 2 * nu));
}

// B^T D B accumulated in the reference's loop order (include/analysis.h:293-319); n =
// 3 npe is a compile-time constant there (dof_per_element), and here too.
template <int n>
void btdb(const double* B, const double* D, double* out) {
  for (int k = 0; k < 6; ++k) {
    const double* bk = B + k * n;
    for (int l = 0; l < 6; ++l) {
      const double dkl = D[6 * k + l];
      const double* bl = B + l * n;
      for (int i = 0; i < n; ++i) {
        const double s = bk[i] * dkl;
        double* row = out + i * n;
        for (int j = 0; j < n; ++j) row[j] += s * bl[j];
      }
    }
  }
}

// y = A x (row-major), cppimpact_gemv NoTrans with alpha = 1, beta = 0 on a zeroed y
// (include/cppimpact_blas.h:9-19).
void gemv(int m, int n, const double* A, const double* x, double* y) {
  for (int i = 0; i < m; i++) {
    y[i] += 0.0;
    for (int j = 0; j < n; j++) y[i] += 1.0 * A[i * n + j] * x[j];
  }
}

// Element stiffness K_e = sum_q w_q detJ_q B^T D B at the given coordinates
// (calculate_f_internal, include/analysis.h:321-378).  pu_jinv reproduces the
// Jinv overwrite of calculate_strain_energy.
template <int NPE>
void element_stiffness_t(const double* xe, const double* D, double* K, bool pu_jinv) {
  constexpr int n = 3 * NPE;
  std::memset(K, 0, sizeof(double) * n * n);
  double B[6 * n], T[n * n];
  for (int q = 0; q < 5; q++) {
    const double* pt = kQ5Pt[q];
    const double w = kQ5W[q];
    double G[30], J[9], Ji[9];
    shape_grad(NPE, pt, G);
    jacobian(NPE, G, xe, J);
    const double detJ = inverse3(J, Ji);
    if (pu_jinv && NPE == 10) {
      double Gp[30], Jp[9];
      shape_grad_pu(pt, Gp);
      jacobian(NPE, Gp, xe, Jp);
      inverse3(Jp, Ji);
    }
    bmatrix(NPE, Ji, G, B);
    std::memset(T, 0, sizeof(T));
    btdb<n>(B, D, T);
    for (int j = 0; j < n * n; j++) K[j] += w * detJ * T[j];
  }
}

void element_stiffness(int npe, const double* xe, const double* D, double* K, bool pu_jinv) {
  if (npe == 4)
    element_stiffness_t<4>(xe, D, K, pu_jinv);
  else
    element_stiffness_t<10>(xe, D, K, pu_jinv);
}

void gather3(int npe, const int* nodes, const double* src, double* dst) {
  for (int j = 0; j < npe; j++)
    for (int k = 0; k < 3; k++) dst[3 * j + k] = src[3 * nodes[j] + k];
}

// Per-element part of update (include/dynamics_kernels.h:75-148) for elements
// [e0, e1): accumulates -f/m into acc, writes per-element strain/stress at xi = 0.
void element_range(const orc_mesh* m, const orc_ref_params* p, const double* xloc0,
                   const double* xloc, const double* dof, const double* mass3, double* acc,
                   double* el_strain, double* el_stress, int e0, int e1) {
  const int npe = m->nodes_per_element, n = 3 * npe;
  double D[36];
  dmatrix(p->E, p->nu, D);
  std::vector<double> K(n * n), B(6 * n);
  double me[30], xe[30], de[30], f[30], x0e[30], tot[30];
  for (int e = e0; e < e1; e++) {
    const int* nodes = m->conn + (size_t)npe * e;
    gather3(npe, nodes, mass3, me);
    gather3(npe, nodes, xloc, xe);
    gather3(npe, nodes, dof, de);
    double rinv[30];
    for (int k = 0; k < n; k++) rinv[k] = 1.0 / me[k];
    element_stiffness(npe, xe, D, K.data(), false);
    std::memset(f, 0, sizeof(f));
    gemv(n, n, K.data(), de, f);
    double ae[30];
    for (int j = 0; j < n; j++) ae[j] = rinv[j] * (-f[j]);
    if (el_strain) {
      // Output-only stress/strain at xi = (0,0,0) from the total displacement
      // (include/dynamics_kernels.h:117-130, include/analysis.h:479-503).
      gather3(npe, nodes, xloc0, x0e);
      for (int j = 0; j < n; j++) tot[j] = de[j] + xe[j] - x0e[j];
      const double pt[3] = {0.0, 0.0, 0.0};
      double G[30], J[9], Ji[9];
      shape_grad(npe, pt, G);
      jacobian(npe, G, xe, J);
      inverse3(J, Ji);
      bmatrix(npe, Ji, G, B.data());
      double eps[6] = {0, 0, 0, 0, 0, 0}, sig[6] = {0, 0, 0, 0, 0, 0};
      gemv(6, n, B.data(), tot, eps);
      gemv(6, 6, D, eps, sig);
      std::memcpy(el_strain + 6 * (size_t)e, eps, sizeof(eps));
      std::memcpy(el_stress + 6 * (size_t)e, sig, sizeof(sig));
    }
    for (int j = 0; j < npe; j++) {
      const int node = nodes[j];
      acc[3 * node] += ae[3 * j];
      acc[3 * node + 1] += ae[3 * j + 1];
      acc[3 * node + 2] += ae[3 * j + 2];
    }
  }
}

}  // namespace

extern "C" int orc_ref_lumped_mass(const orc_mesh* m, double rho, const double* xloc,
                                   double* mass3) {
  // element_mass_matrix (include/analysis.h:136-162) assembled in element order
  // (include/dynamics_kernels.h:36-73).
  const int npe = m->nodes_per_element;
  if (npe != 4 && npe != 10) return -1;
  std::memset(mass3, 0, sizeof(double) * 3 * m->num_nodes);
  double xe[30];
  for (int e = 0; e < m->num_elements; e++) {
    const int* nodes = m->conn + (size_t)npe * e;
    gather3(npe, nodes, xloc, xe);
    double md[10];
    for (int i = 0; i < npe; i++) {
      double mi = 0.0;
      for (int q = 0; q < 5; q++) {
        double G[30], J[9], Ji[9], N[10];
        shape_grad(npe, kQ5Pt[q], G);
        jacobian(npe, G, xe, J);
        const double detJ = inverse3(J, Ji);
        shape(npe, kQ5Pt[q], N);
        mi += N[i] * kQ5W[q] * detJ * rho;
      }
      md[i] = mi;
    }
    for (int j = 0; j < npe; j++) {
      const int node = nodes[j];
      mass3[3 * node] += md[j];
      mass3[3 * node + 1] += md[j];
      mass3[3 * node + 2] += md[j];
    }
  }
  return 0;
}

extern "C" int orc_ref_update(const orc_mesh* m, const orc_ref_params* p, const double* xloc0,
                              const double* xloc, const double* dof, double* acc, double* mass3,
                              double* strains, double* stress, int nthreads) {
  const int N = m->num_nodes, E = m->num_elements, npe = m->nodes_per_element;
  if (npe != 4 && npe != 10) return -1;
  std::memset(acc, 0, sizeof(double) * 3 * N);
  if (mass3[0] == 0.0) orc_ref_lumped_mass(m, p->rho, xloc, mass3);

  std::vector<double> es, ess;
  if (strains || stress) {
    es.resize(6 * (size_t)E);
    ess.resize(6 * (size_t)E);
  }
  double* esp = es.empty() ? nullptr : es.data();
  double* essp = ess.empty() ? nullptr : ess.data();
  if (nthreads <= 1) {
    element_range(m, p, xloc0, xloc, dof, mass3, acc, esp, essp, 0, E);
  } else {
    std::vector<std::vector<double>> part(nthreads, std::vector<double>(3 * (size_t)N, 0.0));
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) {
      const int e0 = (int)((long long)E * t / nthreads), e1 = (int)((long long)E * (t + 1) / nthreads);
      th.emplace_back(element_range, m, p, xloc0, xloc, dof, mass3, part[t].data(), esp, essp, e0, e1);
    }
    for (auto& t : th) t.join();
    for (int t = 0; t < nthreads; t++)
      for (size_t i = 0; i < 3 * (size_t)N; i++) acc[i] += part[t][i];
  }
  if (strains || stress) {
    // last writer wins per node, in element order (include/dynamics_kernels.h:141-147)
    for (int e = 0; e < E; e++)
      for (int j = 0; j < npe; j++) {
        const int node = m->conn[(size_t)npe * e + j];
        for (int k = 0; k < 6; k++) {
          if (strains) strains[6 * node + k] = es[6 * (size_t)e + k];
          if (stress) stress[6 * node + k] = ess[6 * (size_t)e + k];
        }
      }
  }
  // Contact and body force per node (include/dynamics_kernels.h:150-168, wall.h:37-43).
  const double ns = p->wall_normal * p->wall_stiffness;
  for (int i = 0; i < N; i++) {
    const int d = p->wall_dim;
    const double pos = xloc[3 * i + d] + dof[3 * i + d];
    const double dist = (pos - p->wall_location) * p->wall_normal;
    if (dist < 0.0) acc[3 * i + d] += -1 * (1 / mass3[3 * i + d]) * dist * ns;
    acc[3 * i + p->gravity_dim] += p->gravity;
  }
  return 0;
}

extern "C" int orc_ref_solve(const orc_mesh* m, const orc_ref_params* p, const double init_pos[3],
                             const double init_vel[3], double dt, double time_end, int nthreads,
                             double* x_out, double* v_out, double* mass_out, double* acc_out,
                             int* nsteps_out) {
  const int N = m->num_nodes, ndof = 3 * N;
  if (m->nodes_per_element != 4 && m->nodes_per_element != 10) return -1;
  // Dynamics::initialize (include/dynamics.h:99-111)
  std::vector<double> X(ndof), x(ndof), v(ndof), dof(ndof, 0.0), acc(ndof, 0.0), mass(ndof, 0.0);
  for (int i = 0; i < N; i++)
    for (int k = 0; k < 3; k++) {
      v[3 * i + k] = init_vel[k];
      X[3 * i + k] = m->xloc[3 * i + k] + init_pos[k];
    }
  // Dynamics::solve (include/dynamics.h:440-511)
  x = X;
  double time = 0.0;
  orc_ref_update(m, p, X.data(), x.data(), dof.data(), acc.data(), mass.data(), nullptr, nullptr,
                 nthreads);
  for (int i = 0; i < ndof; i++) v[i] += 0.5 * dt * acc[i];
  int steps = 0;
  while (time <= time_end) {
    for (int j = 0; j < ndof; j++) dof[j] = dt * v[j];
    orc_ref_update(m, p, X.data(), x.data(), dof.data(), acc.data(), mass.data(), nullptr, nullptr,
                   nthreads);
    for (int i = 0; i < ndof; i++) {
      x[i] += dof[i];
      v[i] += dt * acc[i];
    }
    time += dt;
    steps++;
  }
  if (x_out) std::memcpy(x_out, x.data(), sizeof(double) * ndof);
  if (v_out) std::memcpy(v_out, v.data(), sizeof(double) * ndof);
  if (mass_out) std::memcpy(mass_out, mass.data(), sizeof(double) * ndof);
  if (acc_out) std::memcpy(acc_out, acc.data(), sizeof(double) * ndof);
  if (nsteps_out) *nsteps_out = steps;
  return 0;
}

extern "C" int orc_ref_debug_strain(const orc_mesh* m, double E, double nu, double alpha,
                                    int def_case, double* energy, double* volume) {
  // Dynamics::debug_strain (include/dynamics.h:303-412) with
  // calculate_strain_energy / calculate_volume (include/analysis.h:384-477).
  const int N = m->num_nodes, npe = m->nodes_per_element, n = 3 * npe;
  if (npe != 4 && npe != 10) return -1;
  std::vector<double> dof(3 * (size_t)N, 0.0);
  for (int i = 0; i < N; i++) {
    const double x = m->xloc[3 * i];
    if (def_case == 0) {
      dof[3 * i] = alpha * x;
      dof[3 * i + 1] = -alpha * x * nu;
      dof[3 * i + 2] = -alpha * x * nu;
    } else if (def_case == 1) {
      dof[3 * i] = alpha * 0.5 * x * x;
      dof[3 * i + 1] = -alpha * 0.5 * x * x * nu;
      dof[3 * i + 2] = -alpha * 0.5 * x * x * nu;
    }
  }
  double D[36];
  dmatrix(E, nu, D);
  std::vector<double> K(n * n);
  double W = 0.0, V = 0.0, xe[30], de[30], Ku[30];
  for (int e = 0; e < m->num_elements; e++) {
    const int* nodes = m->conn + (size_t)npe * e;
    gather3(npe, nodes, m->xloc, xe);
    gather3(npe, nodes, dof.data(), de);
    element_stiffness(npe, xe, D, K.data(), true);
    std::memset(Ku, 0, sizeof(Ku));
    gemv(n, n, K.data(), de, Ku);
    double We = 0.0;
    for (int j = 0; j < n; j++) We += 0.5 * de[j] * Ku[j];
    double Ve = 0.0;
    for (int q = 0; q < 5; q++) {
      double G[30], J[9], Ji[9];
      shape_grad(npe, kQ5Pt[q], G);
      jacobian(npe, G, xe, J);
      Ve += kQ5W[q] * inverse3(J, Ji);
    }
    W += We;
    V += Ve;
  }
  *energy = W;
  *volume = V;
  return 0;
}
