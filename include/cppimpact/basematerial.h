// basematerial.h -- drop-in for include/basematerial.h (BaseMaterial{E, rho, nu}).
#pragma once
#include <string>

template <typename T, int dof_per_node>
class BaseMaterial {
 public:
  int ndof = dof_per_node;
  std::string name;
  std::string type;
  T E;
  T rho;
  T nu;

  BaseMaterial(std::string type, T E, T rho, T nu, std::string name = "Material")
      : name(name), type(type), E(E), rho(rho), nu(nu) {}
  virtual ~BaseMaterial() {}

  // J2 parameters; zero for a purely elastic material.
  virtual T get_beta() const { return T(0); }
  virtual T get_H() const { return T(0); }
  virtual T get_Y0() const { return T(0); }
};
