// wall.h -- drop-in for include/wall.h: Wall<T, dim, Basis>(name, location, stiffness,
// slave_node_indices, num_slave_nodes, normal).  The GPU solver receives it as the
// plane normal = normal * e_dim, offset = normal * location (ci_wall).
#pragma once
#include <string>

#include "cppimpact_defs.h"

template <typename T, int dim, class Basis>
class Wall {
 public:
  std::string name;
  T location;
  T stiffness;
  int* slave_node_indices;
  int num_slave_nodes;
  int normal;
  T norm_stiffness;

  Wall(std::string name, T location, T stiffness, int* slave_node_indices, int num_slave_nodes,
       int normal)
      : name(name),
        location(location),
        stiffness(stiffness),
        slave_node_indices(slave_node_indices),
        num_slave_nodes(num_slave_nodes),
        normal(normal) {
    norm_stiffness = normal * stiffness;
  }
  ~Wall() {}

  // Penalty acceleration on one node (host version of the reference's rule).
  CPPIMPACT_FUNCTION void detect_contact(T* global_acc, int node_idx, T* node_pos, T* node_mass) {
    T d = (node_pos[dim] - location) * normal;
    if (d < 0.0) global_acc[3 * node_idx + dim] += -1 * (1 / node_mass[dim]) * d * norm_stiffness;
  }

  ci_wall as_ci() const {
    ci_wall w;
    w.normal[0] = w.normal[1] = w.normal[2] = 0.0;
    w.normal[dim] = (double)normal;
    w.offset = (double)normal * (double)location;
    w.stiffness = (double)stiffness;
    return w;
  }
};
