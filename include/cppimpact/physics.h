// physics.h -- drop-in for include/physics.h: the Physics template argument and the
// 3x3 helpers (det3x3, inv3x3) on the host.  NeohookeanPhysics is only ever used for
// its dof_per_node on the reference's hot path.
#pragma once
#include <cmath>

#include "cppimpact_defs.h"

template <typename T>
inline T det3x3(const T A[]) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

template <typename T>
inline T inv3x3(const T A[], T Ainv[]) {
  const T det = det3x3(A);
  const T r = T(1) / det;
  Ainv[0] = (A[4] * A[8] - A[5] * A[7]) * r;
  Ainv[1] = (A[2] * A[7] - A[1] * A[8]) * r;
  Ainv[2] = (A[1] * A[5] - A[2] * A[4]) * r;
  Ainv[3] = (A[5] * A[6] - A[3] * A[8]) * r;
  Ainv[4] = (A[0] * A[8] - A[2] * A[6]) * r;
  Ainv[5] = (A[2] * A[3] - A[0] * A[5]) * r;
  Ainv[6] = (A[3] * A[7] - A[4] * A[6]) * r;
  Ainv[7] = (A[1] * A[6] - A[0] * A[7]) * r;
  Ainv[8] = (A[0] * A[4] - A[1] * A[3]) * r;
  return det;
}

template <typename T>
class NeohookeanPhysics {
 public:
  static const int dof_per_node = 3;
};
