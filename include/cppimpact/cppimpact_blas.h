// cppimpact_blas.h -- drop-in for include/cppimpact_blas.h (row-major gemv helper).
#pragma once
enum class MatOp { NoTrans, Trans };

template <typename T, MatOp op>
void cppimpact_gemv(const int m, const int n, const T alpha, const T* a, const T* x, const T beta,
                    T* y) {
  if (op == MatOp::NoTrans) {
    for (int i = 0; i < m; i++) {
      T s = T(0);
      for (int j = 0; j < n; j++) s += a[i * n + j] * x[j];
      y[i] = beta * y[i] + alpha * s;
    }
  } else {
    for (int i = 0; i < n; i++) {
      T s = T(0);
      for (int j = 0; j < m; j++) s += a[j * n + i] * x[j];
      y[i] = beta * y[i] + alpha * s;
    }
  }
}
