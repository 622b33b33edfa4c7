// mesh.h -- drop-in for include/mesh.h: Mesh<T, nodes_per_element> with the same public
// fields; load_mesh parses the .inp file in libcppimpact_gb300.so (ci_mesh_load_inp),
// same subset and 1-based -> 0-based id mapping as the reference (include/mesh.h:57-267).
#pragma once
#include <string>
#include <vector>

#include "cppimpact_defs.h"

template <typename T, int nodes_per_element>
class Mesh {
 public:
  int num_elements = 0, num_nodes = 0, num_node_sets = 0, num_fixed_nodes = 0,
      num_slave_nodes = 0;
  int *element_nodes = nullptr, *node_set_starts = nullptr, *node_set_indices = nullptr,
      *fixed_nodes = nullptr, *slave_nodes = nullptr;
  T* xloc = nullptr;
  std::vector<std::string> node_set_names;

  Mesh() {}
  ~Mesh() { release(); }
  Mesh(const Mesh&) = delete;
  Mesh& operator=(const Mesh&) = delete;

  // 0 on success, 1 when the file cannot be opened or parsed.
  int load_mesh(std::string filename) {
    ci_mesh m;
    const int rc = ci_mesh_load_inp(filename.c_str(), nodes_per_element, &m);
    if (rc != CI_OK) {
      std::cerr << "Failed to open file: " << filename << std::endl;
      return 1;
    }
    release();
    num_nodes = m.num_nodes;
    num_elements = m.num_elements;
    xloc = new T[3 * (size_t)num_nodes];
    for (size_t i = 0; i < 3 * (size_t)num_nodes; i++) xloc[i] = (T)m.xloc[i];
    element_nodes = new int[(size_t)nodes_per_element * num_elements];
    std::memcpy(element_nodes, m.element_nodes, sizeof(int) * nodes_per_element * (size_t)num_elements);
    num_slave_nodes = m.num_slave_nodes;
    num_fixed_nodes = m.num_fixed_nodes;
    slave_nodes = new int[num_slave_nodes + 1];
    fixed_nodes = new int[num_fixed_nodes + 1];
    std::memcpy(slave_nodes, m.slave_nodes, sizeof(int) * num_slave_nodes);
    std::memcpy(fixed_nodes, m.fixed_nodes, sizeof(int) * num_fixed_nodes);
    if (num_slave_nodes == 0)
      std::printf("No slave node sets found. Walls will have no effect on simulation.\n");
    ci_mesh_free(&m);
    return 0;
  }

  ci_mesh as_ci(std::vector<double>* xbuf) const {
    xbuf->assign(xloc, xloc + 3 * (size_t)num_nodes);
    ci_mesh m;
    m.num_nodes = num_nodes;
    m.num_elements = num_elements;
    m.nodes_per_element = nodes_per_element;
    m.xloc = xbuf->data();
    m.element_nodes = element_nodes;
    m.num_slave_nodes = num_slave_nodes;
    m.slave_nodes = slave_nodes;
    m.num_fixed_nodes = num_fixed_nodes;
    m.fixed_nodes = fixed_nodes;
    return m;
  }

 private:
  void release() {
    delete[] element_nodes;
    delete[] node_set_starts;
    delete[] node_set_indices;
    delete[] xloc;
    delete[] fixed_nodes;
    delete[] slave_nodes;
    element_nodes = node_set_starts = node_set_indices = fixed_nodes = slave_nodes = nullptr;
    xloc = nullptr;
  }
};
