// elastoplastic.h -- drop-in for include/elastoplastic.h.  Same constructor
// (E, rho, nu, beta, H, Y0, name); the J2 parameters the reference stores but never
// reads are exposed through get_beta/get_H/get_Y0 and used by the J2 mode.
#pragma once
#include <stdexcept>

#include "basematerial.h"

template <typename T, int dof_per_node>
class Elastoplastic : public BaseMaterial<T, dof_per_node> {
 public:
  Elastoplastic(T E, T rho, T nu, T beta, T H, T Y0, std::string name = "Material")
      : BaseMaterial<T, dof_per_node>("InfinitesimalElastoplastic", E, rho, nu, name),
        beta(beta),
        H(H),
        Y0_initial_yield_stress(Y0) {}
  virtual ~Elastoplastic() {}

  T get_beta() const override { return beta; }
  T get_H() const override { return H; }
  T get_Y0() const override { return Y0_initial_yield_stress; }

 protected:
  T beta;
  T H;
  T Y0_initial_yield_stress;
};
