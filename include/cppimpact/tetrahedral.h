// tetrahedral.h -- drop-in for include/tetrahedral.h: the basis and quadrature types
// used as template arguments of Dynamics/FEAnalysis.  The GPU path uses its own rules
// (1-point tet4, 4-point Gauss tet10); these host helpers give the element's shape
// functions in the reference's node order (corners xi, eta, 1-xi-eta-zeta, zeta for
// tet10; 1-xi-eta-zeta, xi, eta, zeta for tet4; CalculiX edge order).
#pragma once
#include "cppimpact_defs.h"

// 5-point rule of degree 3 on the unit tetrahedron (the reference truncates the
// constants to 11 digits; these are exact).
class TetrahedralQuadrature5pts {
 public:
  static const int num_quadrature_pts = 5;
  template <typename T>
  static T get_quadrature_pt(int k, T pt[]) {
    const T a = T(1) / T(6), b = T(0.5);
    const T P[5][3] = {{0.25, 0.25, 0.25}, {a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
    if (k < 0 || k > 4) return T(0);
    pt[0] = P[k][0];
    pt[1] = P[k][1];
    pt[2] = P[k][2];
    return k == 0 ? T(-2) / T(15) : T(3) / T(40);
  }
};

// 4-point Gauss rule of degree 2.
class TetrahedralQuadrature4pts {
 public:
  static const int num_quadrature_pts = 4;
  template <typename T>
  static T get_quadrature_pt(int k, T pt[]) {
    const T a = T(0.58541019662496845446), b = T(0.13819660112501051518);
    if (k < 0 || k > 3) return T(0);
    pt[0] = k == 1 ? a : b;
    pt[1] = k == 2 ? a : b;
    pt[2] = k == 3 ? a : b;
    return T(1) / T(24);
  }
};

template <typename T>
class TetrahedralBasisLinear {
 public:
  static constexpr int spatial_dim = 3;
  static constexpr int nodes_per_element = 4;
  static void eval_basis(const T pt[], T N[]) {
    N[0] = T(1) - pt[0] - pt[1] - pt[2];
    N[1] = pt[0];
    N[2] = pt[1];
    N[3] = pt[2];
  }
  static void eval_basis_grad(const T*, T Nxi[]) {
    const T g[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < 12; i++) Nxi[i] = g[i];
  }
};

template <typename T>
class TetrahedralBasisQuadratic {
 public:
  static constexpr int spatial_dim = 3;
  static constexpr int nodes_per_element = 10;
  static void eval_basis(const T pt[], T N[]) {
    const T L[4] = {pt[0], pt[1], T(1) - pt[0] - pt[1] - pt[2], pt[2]};
    const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
    for (int c = 0; c < 4; c++) N[c] = L[c] * (T(2) * L[c] - T(1));
    for (int k = 0; k < 6; k++) N[4 + k] = T(4) * L[ea[k]] * L[eb[k]];
  }
  static void eval_basis_grad(const T pt[], T Nxi[]) {
    const T L[4] = {pt[0], pt[1], T(1) - pt[0] - pt[1] - pt[2], pt[2]};
    const T dL[4][3] = {{1, 0, 0}, {0, 1, 0}, {-1, -1, -1}, {0, 0, 1}};
    const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
    for (int c = 0; c < 4; c++)
      for (int j = 0; j < 3; j++) Nxi[3 * c + j] = (T(4) * L[c] - T(1)) * dL[c][j];
    for (int k = 0; k < 6; k++)
      for (int j = 0; j < 3; j++)
        Nxi[3 * (4 + k) + j] = T(4) * (L[ea[k]] * dL[eb[k]][j] + L[eb[k]] * dL[ea[k]][j]);
  }
};
