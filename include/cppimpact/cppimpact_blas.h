// cppimpact_blas.h -- drop-in for include/cppimpact_blas.h (row-major gemv helper).
//
// Semantics are kept exactly as the reference defines them (include/cppimpact_blas.h:9-29),
// which is NOT the BLAS convention: every y[i] first gets beta ADDED to it, then the
// products alpha * a * x are accumulated into y[i] one term at a time.  The result is
// y_i <- y_i + beta + sum_j alpha a_ij x_j; with beta = 0 and y zeroed beforehand (how
// the reference's analysis code calls it) this is y = alpha op(A) x.
#pragma once
enum class MatOp { NoTrans, Trans };

template <typename T, MatOp op>
void cppimpact_gemv(const int m, const int n, const T alpha, const T* a, const T* x, const T beta,
                    T* y) {
  // NoTrans: y has m entries, row i of A is a[i*n .. i*n+n); Trans: y has n entries,
  // column i of A (a[j*n + i], j < m) is the row used.
  const int rows = op == MatOp::NoTrans ? m : n;
  const int len = op == MatOp::NoTrans ? n : m;
  for (int i = 0; i < rows; i++) {
    T acc = y[i] + beta;
    for (int j = 0; j < len; j++) {
      const T aij = op == MatOp::NoTrans ? a[i * n + j] : a[j * n + i];
      acc += alpha * aij * x[j];
    }
    y[i] = acc;
  }
}
