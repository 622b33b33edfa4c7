// dynamics.h -- drop-in for include/dynamics.h.
//
// Dynamics<T, Basis, Analysis, Quadrature>(Mesh*, BaseMaterial*, Wall*) with
// initialize(pos, vel), solve(dt, time_end, export_interval) and debug_strain(alpha,
// case), and the public host arrays of the reference (global_xloc, vel, global_mass,
// global_acc, global_strains, global_stress, vel_i, timestep).  The time loop runs on
// the GPU inside libcppimpact_gb300.so; the host arrays are filled at each export
// step and at the end of solve.  The VTK files carry the reference's fields in its
// order (velocity, strain1/2, stress1/2, acceleration, mass); tet10 cells are written
// as VTK_QUADRATIC_TETRA (24) where the reference writes VTK_TETRA (10) for both.
//
// force_law selects the constitutive model: CI_MODE_REFCOMPAT (default) reproduces the
// reference's incremental force K_e(x_n) (dt v) with row-sum mass; CI_MODE_J2 uses
// the material's J2 parameters (Elastoplastic::get_Y0, get_H) with HRZ mass.
#pragma once
#include <cmath>
#include <algorithm>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <vector>

#include "basematerial.h"
#include "cppimpact_utils.h"
#include "mesh.h"
#include "wall.h"

template <typename T, class Basis, class Analysis, class Quadrature>
class Dynamics {
  static_assert(sizeof(T) == sizeof(double), "the GPU solver's nodal state is FP64");

 public:
  int* reduced_nodes = nullptr;
  int reduced_dofs_size = 0;
  int ndof;
  static constexpr int nodes_per_element = Basis::nodes_per_element;
  static constexpr int spatial_dim = Basis::spatial_dim;
  static constexpr int dof_per_node = spatial_dim;
  static constexpr int num_quadrature_pts = Quadrature::num_quadrature_pts;

  Mesh<T, nodes_per_element>* mesh;
  BaseMaterial<T, dof_per_node>* material;
  Wall<T, 2, Basis>* wall;
  T* global_xloc;
  T* vel;
  T* global_strains;
  T* global_stress;
  T* global_dof;
  T* global_acc;
  T* global_mass;
  T* vel_i;
  int timestep = 0;
  double time = 0.0;
  int force_law = CI_MODE_REFCOMPAT;
  std::string output_dir = "../cpu_output";

  Dynamics(Mesh<T, nodes_per_element>* input_mesh, BaseMaterial<T, dof_per_node>* input_material,
           Wall<T, 2, Basis>* input_wall = nullptr)
      : mesh(input_mesh), material(input_material), wall(input_wall) {
    ndof = mesh->num_nodes * dof_per_node;
    global_xloc = new T[ndof]();
    vel = new T[ndof]();
    global_strains = new T[6 * (size_t)mesh->num_nodes]();
    global_stress = new T[6 * (size_t)mesh->num_nodes]();
    global_dof = new T[ndof]();
    global_acc = new T[ndof]();
    global_mass = new T[ndof]();
    vel_i = new T[ndof]();
  }

  ~Dynamics() {
    if (solver_) ci_destroy(solver_);
    delete[] reduced_nodes;
    delete[] vel;
    delete[] global_xloc;
    delete[] global_strains;
    delete[] global_stress;
    delete[] global_dof;
    delete[] global_acc;
    delete[] global_mass;
    delete[] vel_i;
  }

  // Move the mesh by init_position and give every node init_velocity
  // (include/dynamics.h:99-111).
  void initialize(T init_position[dof_per_node], T init_velocity[dof_per_node]) {
    for (int i = 0; i < mesh->num_nodes; i++)
      for (int k = 0; k < 3; k++) {
        vel[3 * i + k] = init_velocity[k];
        mesh->xloc[3 * i + k] += init_position[k];
      }
  }

  // Staggered central difference from the mesh positions and the current vel array:
  // mass, a0, v += dt/2 a0, then steps while time <= time_end (include/dynamics.h:414-512).
  void solve(double dt, double time_end, int export_interval) {
    ensure_solver();
    std::memcpy(global_xloc, mesh->xloc, sizeof(T) * ndof);
    cppimpact_gb300::check(ci_set_state(solver_, global_xloc, vel), "ci_set_state");
    cppimpact_gb300::check(ci_start(solver_, dt), "ci_start");
    long long total = 0;
    for (double t = 0.0; t <= time_end; t += dt) total++;
    time = 0.0;
    long long done = 0;
    // As in the reference's loop, the step with 0-based index t is exported (after it
    // ran) when t % export_interval == 0; export_interval <= 0 exports nothing.
    while (done < total) {
      long long n = std::min<long long>(total - done, INT_MAX);
      if (export_interval > 0)
        n = std::min<long long>(n, (export_interval - timestep % export_interval) % export_interval + 1);
      cppimpact_gb300::check(ci_step(solver_, (int)n), "ci_step");
      done += n;
      timestep += (int)n;
      time += n * dt;
      if (export_interval > 0 && (timestep - 1) % export_interval == 0) {
        fetch(dt);
        export_to_vtk(timestep - 1, vel_i, global_acc, global_mass);
      }
    }
    fetch(dt);
  }

  // Total strain energy and volume for a prescribed displacement (include/dynamics.h:303-412).
  void debug_strain(const T alpha, const int def_case) {
    ensure_solver();
    std::vector<double> u(ndof, 0.0);
    for (int i = 0; i < mesh->num_nodes; i++) {
      const double x = mesh->xloc[3 * i];
      const double g = def_case == 0 ? x : (def_case == 1 ? 0.5 * x * x : 0.0);
      u[3 * i] = alpha * g;
      u[3 * i + 1] = -alpha * g * material->nu;
      u[3 * i + 2] = -alpha * g * material->nu;
    }
    double W = 0.0, V = 0.0;
    cppimpact_gb300::check(ci_strain_energy(solver_, u.data(), &W, &V), "ci_strain_energy");
    last_strain_energy = W;
    last_volume = V;
    std::printf("Total Strain Energy = %f\n", W);
    std::printf("Total Volume = %f\n", V);
    for (int i = 0; i < ndof; i++) global_xloc[i] = mesh->xloc[i] + u[i];
  }

  // Legacy ASCII VTK of the current state (include/dynamics.h:113-254).
  void export_to_vtk(int step, T* vel_out, T* acc_out, T* mass_out) {
    const std::string fn = output_dir + "/simulation_" + std::to_string(step) + ".vtk";
    std::ofstream f(fn);
    if (!f.is_open()) {
      std::cerr << "Failed to open " << fn << std::endl;
      return;
    }
    f << "# vtk DataFile Version 3.0\nFEA simulation data\nASCII\nDATASET UNSTRUCTURED_GRID\n";
    f << "POINTS " << mesh->num_nodes << " float\n" << std::fixed << std::setprecision(6);
    for (int i = 0; i < mesh->num_nodes; i++)
      f << global_xloc[3 * i] << " " << global_xloc[3 * i + 1] << " " << global_xloc[3 * i + 2] << "\n";
    f << "CELLS " << mesh->num_elements << " " << mesh->num_elements * (nodes_per_element + 1) << "\n";
    for (int e = 0; e < mesh->num_elements; e++) {
      f << nodes_per_element;
      for (int j = 0; j < nodes_per_element; j++) f << " " << mesh->element_nodes[nodes_per_element * e + j];
      f << "\n";
    }
    f << "CELL_TYPES " << mesh->num_elements << "\n";
    for (int e = 0; e < mesh->num_elements; e++) f << (nodes_per_element == 10 ? 24 : 10) << "\n";
    f << "POINT_DATA " << mesh->num_nodes << "\n";
    auto vec = [&](const char* name, const T* a) {
      f << "VECTORS " << name << " double\n";
      for (int i = 0; i < mesh->num_nodes; i++)
        f << a[3 * i] << " " << a[3 * i + 1] << " " << a[3 * i + 2] << "\n";
    };
    // six-component fields as two 3-vectors each (include/dynamics.h:194-225)
    auto half = [&](const char* name, const T* a, int off) {
      f << "VECTORS " << name << " double\n";
      for (int i = 0; i < mesh->num_nodes; i++)
        f << a[6 * i + off] << " " << a[6 * i + off + 1] << " " << a[6 * i + off + 2] << "\n";
    };
    vec("velocity", vel_out);
    half("strain1", global_strains, 0);
    half("strain2", global_strains, 3);
    half("stress1", global_stress, 0);
    half("stress2", global_stress, 3);
    vec("acceleration", acc_out);
    vec("mass", mass_out);
  }

  double last_strain_energy = 0.0, last_volume = 0.0;

 private:
  ci_solver* solver_ = nullptr;

  void ensure_solver() {
    if (solver_) return;
    std::vector<double> xb;
    const ci_mesh m = mesh->as_ci(&xb);
    ci_material mat;
    mat.E = material->E;
    mat.nu = material->nu;
    mat.rho = material->rho;
    mat.sigma_y0 = force_law == CI_MODE_J2 ? material->get_Y0() : 0.0;
    mat.H = material->get_H();
    mat.beta = 0.0;
    ci_wall w;
    if (wall) {
      w = wall->as_ci();
    } else {
      w.normal[0] = w.normal[1] = 0.0;
      w.normal[2] = 1.0;
      w.offset = -1e300;
      w.stiffness = 0.0;
    }
    ci_options o;
    ci_default_options(&o);
    o.mode = force_law;
    o.lumping = force_law == CI_MODE_REFCOMPAT ? CI_LUMP_ROWSUM : CI_LUMP_HRZ;
    cppimpact_gb300::check(ci_create(&m, &mat, &w, &o, &solver_), "ci_create");
  }

  // Host arrays from the GPU state: positions, half-step velocity, masses, the last
  // step's acceleration, the full-step velocity vel - dt/2 acc (include/dynamics.h:501)
  // and the nodal strain/stress fields (include/dynamics_kernels.h:117-147).
  void fetch(double dt) {
    std::vector<double> m(mesh->num_nodes);
    cppimpact_gb300::check(ci_get_state(solver_, global_xloc, vel, m.data(), nullptr, nullptr, nullptr),
                           "ci_get_state");
    cppimpact_gb300::check(ci_get_nodal_fields(solver_, global_acc, global_strains, global_stress),
                           "ci_get_nodal_fields");
    for (int i = 0; i < mesh->num_nodes; i++)
      for (int k = 0; k < 3; k++) {
        global_mass[3 * i + k] = m[i];
        vel_i[3 * i + k] = vel[3 * i + k] - 0.5 * dt * global_acc[3 * i + k];
      }
  }
};
