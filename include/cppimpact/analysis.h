// analysis.h -- drop-in for include/analysis.h.  FEAnalysis<T, Basis, Quadrature,
// Physics> carries the element constants the reference's templates use; the element
// computations themselves (mass, internal force, strain energy) run in
// libcppimpact_gb300.so (ci_lumped_mass, ci_internal_force, ci_strain_energy).
#pragma once
#include "basematerial.h"
#include "cppimpact_blas.h"
#include "cppimpact_defs.h"
#include "mesh.h"
#include "physics.h"
#include "simulation_config.h"
#include "tetrahedral.h"

template <typename T, class Basis, class Quadrature, class Physics>
class FEAnalysis {
 public:
  static constexpr int spatial_dim = 3;
  static constexpr int nodes_per_element = Basis::nodes_per_element;
  static constexpr int num_quadrature_pts = Quadrature::num_quadrature_pts;
  static constexpr int dof_per_node = Physics::dof_per_node;
  static constexpr int dof_per_element = dof_per_node * nodes_per_element;

  // Gather nodal ndof-vectors of one element (include/analysis.h:56-66).
  template <int ndof>
  static void get_element_dof(const int nodes[], const T dof[], T element_dof[]) {
    for (int j = 0; j < nodes_per_element; j++)
      for (int k = 0; k < dof_per_node; k++) element_dof[dof_per_node * j + k] = dof[ndof * nodes[j] + k];
  }
};
