// ref_driver.cu -- TEST INFRASTRUCTURE ONLY.
//
// Harness around the UNMODIFIED reference headers (include path points at the
// reference checkout; nothing is copied).  Built by oracle/Makefile into
// oracle/_ref/ (git-ignored) with nvcc as the host compiler, once with
// -DUSE_LINEAR_BASIS and once with -DUSE_QUADRATIC_BASIS.  Used only to produce the
// golden fixtures under tests/golden/ and to validate the restatement in
// oracle/ref_port.cpp.
//
//   ref_driver solve  <mesh.inp> <out> E rho nu wall_loc wall_k wall_normal vx vy vz dt t_end
//       Dynamics::initialize + Dynamics::solve (include/dynamics.h:99, 414); writes
//       <out>.x <out>.v <out>.mass <out>.acc (raw float64, 3N each) and prints nsteps.
//   ref_driver update <mesh.inp> <dof.f64> <out> E rho nu wall_loc wall_k wall_normal
//       one call of update() (include/dynamics_kernels.h:8) from the mesh positions
//       with the given increment; writes <out>.acc <out>.mass.
//   ref_driver strain <mesh.inp> <case> E nu alpha
//       total strain energy and volume of Dynamics::debug_strain
//       (include/dynamics.h:303-412), printed with 17 significant digits.
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

// clang-format off
#include "include/simulation_config.h"
#include "include/analysis.h"
// clang-format on
#include "include/dynamics.h"
#include "include/elastoplastic.h"
#include "include/wall.h"

static void write_f64(const std::string& path, const double* a, size_t n) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fwrite(a, sizeof(double), n, f);
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_driver solve|update|strain <mesh.inp> ...\n");
    return 2;
  }
  const std::string mode = argv[1];
  Mesh<T, Basis::nodes_per_element> mesh;
  if (mesh.load_mesh(argv[2]) != 0) return 1;

  if (mode == "strain") {
    const int def_case = std::atoi(argv[3]);
    const double E = std::atof(argv[4]), nu = std::atof(argv[5]), alpha = std::atof(argv[6]);
    Elastoplastic<T, 3> mat(E, 2700.0, nu, 0.0, 10.0, 1.0, "m");
    const int npe = Basis::nodes_per_element;
    std::vector<double> dof(3 * mesh.num_nodes, 0.0);
    for (int i = 0; i < mesh.num_nodes; i++) {
      const double x = mesh.xloc[3 * i];
      if (def_case == 0) {
        dof[3 * i] = alpha * x;
        dof[3 * i + 1] = -alpha * x * mat.nu;
        dof[3 * i + 2] = -alpha * x * mat.nu;
      } else {
        dof[3 * i] = alpha * 0.5 * x * x;
        dof[3 * i + 1] = -alpha * 0.5 * x * x * mat.nu;
        dof[3 * i + 2] = -alpha * 0.5 * x * x * mat.nu;
      }
    }
    double W = 0.0, V = 0.0;
    std::vector<double> xe(3 * npe), de(3 * npe);
    for (int e = 0; e < mesh.num_elements; e++) {
      const int* nodes = mesh.element_nodes + npe * e;
      Analysis::get_element_dof<3>(nodes, mesh.xloc, xe.data());
      Analysis::get_element_dof<3>(nodes, dof.data(), de.data());
      W += Analysis::calculate_strain_energy(xe.data(), de.data(), &mat);
      V += Analysis::calculate_volume(xe.data(), de.data(), &mat);
    }
    std::printf("energy %.17g\nvolume %.17g\n", W, V);
    return 0;
  }

  const int a0 = mode == "solve" ? 4 : 5;
  const double E = std::atof(argv[a0]), rho = std::atof(argv[a0 + 1]), nu = std::atof(argv[a0 + 2]);
  const double wall_loc = std::atof(argv[a0 + 3]), wall_k = std::atof(argv[a0 + 4]);
  const int wall_normal = std::atoi(argv[a0 + 5]);
  Elastoplastic<T, 3> mat(E, rho, nu, 0.0, 10.0, 1.0, "m");
  Wall<T, 2, Basis> wall("wall", wall_loc, wall_k, mesh.slave_nodes, mesh.num_slave_nodes,
                         wall_normal);
  const int ndof = 3 * mesh.num_nodes;

  if (mode == "solve") {
    const std::string out = argv[3];
    T pos[3] = {0.0, 0.0, 0.0};
    T vel[3] = {std::atof(argv[a0 + 6]), std::atof(argv[a0 + 7]), std::atof(argv[a0 + 8])};
    const double dt = std::atof(argv[a0 + 9]), t_end = std::atof(argv[a0 + 10]);
    Dynamics<T, Basis, Analysis, Quadrature> dyn(&mesh, &mat, &wall);
    dyn.timestep = 1;  // never initialised by the reference; 1 keeps exports off
    dyn.initialize(pos, vel);
    dyn.solve(dt, t_end, INT_MAX);
    write_f64(out + ".x", dyn.global_xloc, ndof);
    write_f64(out + ".v", dyn.vel, ndof);
    write_f64(out + ".mass", dyn.global_mass, ndof);
    write_f64(out + ".acc", dyn.global_acc, ndof);
    std::fprintf(stderr, "nsteps %d\n", dyn.timestep - 1);
    return 0;
  }
  if (mode == "update") {
    std::vector<double> dof(ndof);
    FILE* f = std::fopen(argv[3], "rb");
    if (!f || std::fread(dof.data(), sizeof(double), ndof, f) != (size_t)ndof) return 3;
    std::fclose(f);
    const std::string out = argv[4];
    std::vector<double> vel(ndof, 0.0), acc(ndof, 0.0), mass(ndof, 0.0),
        strains(6 * mesh.num_nodes, 0.0), stress(6 * mesh.num_nodes, 0.0);
    std::vector<double> xloc(mesh.xloc, mesh.xloc + ndof);
    update<T, 3, Basis::nodes_per_element, Basis, Analysis>(
        mesh.num_nodes, mesh.num_elements, ndof, 1e-7, &mat, &wall, &mesh, mesh.element_nodes,
        vel.data(), xloc.data(), dof.data(), acc.data(), mass.data(), strains.data(),
        stress.data(), 0.0);
    write_f64(out + ".acc", acc.data(), ndof);
    write_f64(out + ".mass", mass.data(), ndof);
    return 0;
  }
  std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
