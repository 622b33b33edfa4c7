// simulation_config.h -- drop-in for include/simulation_config.h: the compile-time
// configuration the reference's drivers rely on (T, Basis, Quadrature, Physics, Analysis).
#pragma once
#include "physics.h"
#include "tetrahedral.h"

template <typename T, class Basis, class Quadrature, class Physics>
class FEAnalysis;

using T = double;

#if defined(USE_QUADRATIC_BASIS)
using Basis = TetrahedralBasisQuadratic<T>;
#else
using Basis = TetrahedralBasisLinear<T>;
#endif

using Quadrature = TetrahedralQuadrature5pts;
using Physics = NeohookeanPhysics<T>;
using Analysis = FEAnalysis<T, Basis, Quadrature, Physics>;
constexpr int dof_per_node = 3;
