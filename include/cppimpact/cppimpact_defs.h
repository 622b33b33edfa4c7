// cppimpact_defs.h -- drop-in for the reference's include/cppimpact_defs.h.
// CPPIMPACT_FUNCTION marks functions usable on host and device (include/cppimpact_defs.h:10,31);
// in the drop-in headers all element math runs inside libcppimpact_gb300.so, so it is
// a plain host qualifier unless compiled by nvcc.
#pragma once
#include <climits>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <stdexcept>

#include "../cppimpact_gb300.h"

#ifdef __CUDACC__
#define CPPIMPACT_FUNCTION __host__ __device__
#else
#define CPPIMPACT_FUNCTION
#endif

namespace cppimpact_gb300 {
// Throws with the library's message when a C-ABI call fails (the reference has no
// error channel; failures there surface as NaNs or crashes).
inline void check(int rc, const char* what) {
  if (rc != CI_OK) {
    std::fprintf(stderr, "cppimpact_gb300: %s failed (%d): %s\n", what, rc, ci_last_error());
    throw std::runtime_error(std::string(what) + ": " + ci_last_error());
  }
}
}  // namespace cppimpact_gb300
