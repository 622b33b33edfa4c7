// ci_mlp.cu -- the surrogate's MLP (n_in -> H -> H -> n_out, tanh hidden layers):
// forward, backward and Adam on the GPU, every matrix product through ci_gemm_bf16
// (BF16 operands, FP32 accumulation), FP32 master weights, fixed-order reductions.
//
// Parameters, in the order ci_mlp_get_params / set_params use:
//   W1 [n_in x H], b1 [H], W2 [H x H], b2 [H], W3 [H x n_out], b3 [n_out]
// (row-major; a layer computes Z = X W + b).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "../../include/cppimpact_gb300.h"

namespace ci {
int set_last_error(int code, const char* msg);
}

namespace {

using bf16 = __nv_bfloat16;

#define CM_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return ci::set_last_error(CI_ERR_CUDA, (std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
  } while (0)

#define CM_OK(call)              \
  do {                           \
    const int rc_ = (call);      \
    if (rc_ != CI_OK) return rc_; \
  } while (0)

__global__ void k_to_bf16(const float* in, bf16* out, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16(in[i]);
}

// dY = scale (Y - T) (scale = 2 / (rows * cols)); per-block partial sum of (Y - T)^2
__global__ void k_mse_grad(const float* Y, const float* T, float* dY, bf16* dYb, long long n,
                           float scale, double* part) {
  __shared__ double red[256];
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double s = 0.0;
  if (i < n) {
    const float d = Y[i] - T[i];
    dY[i] = scale * d;
    dYb[i] = __float2bfloat16(scale * d);
    s = (double)d * d;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// dZ = dH (1 - H^2)
__global__ void k_tanh_back(const float* dH, const float* H, float* dZ, bf16* dZb, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) {
    const float v = dH[i] * (1.f - H[i] * H[i]);
    dZ[i] = v;
    dZb[i] = __float2bfloat16(v);
  }
}

// column sums of a [rows x cols] matrix, one thread per column, rows in order
__global__ void k_colsum(const float* A, int rows, int cols, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; r++) s += A[(size_t)r * cols + c];
  out[c] = s;
}

// Adam (Kingma & Ba 2015) on FP32 master weights; refreshes the BF16 copy
__global__ void k_adam(float* p, const float* g, float* m, float* v, bf16* pb, long long n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / c1, vh = vi / c2;
  const float pi = p[i] - lr * mh / (sqrtf(vh) + eps);
  p[i] = pi;
  if (pb) pb[i] = __float2bfloat16(pi);
}

// rows of X picked by idx -> Xb (BF16) and the matching rows of T
__global__ void k_gather_rows(const float* X, const float* T, const int* idx, int rows, int nx, int nt,
                              bf16* Xb, float* Tb) {
  const int r = blockIdx.x;
  if (r >= rows) return;
  const int s = idx[r];
  for (int j = threadIdx.x; j < nx; j += blockDim.x) Xb[(size_t)r * nx + j] = __float2bfloat16(X[(size_t)s * nx + j]);
  for (int j = threadIdx.x; j < nt; j += blockDim.x) Tb[(size_t)r * nt + j] = T[(size_t)s * nt + j];
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    return count ? cudaMalloc(&p, sizeof(T) * count) : cudaSuccess;
  }
};

inline unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

struct ci_mlp {
  int n_in = 0, H = 0, n_out = 0;
  long long np = 0;           // parameter count
  long long off[6] = {0};     // W1 b1 W2 b2 W3 b3 offsets in the flat arrays
  DBuf<float> p, g, m, v;     // FP32 master params, grads, Adam moments
  DBuf<bf16> pb;              // BF16 copy of the parameters
  DBuf<int> err;
  long long step = 0;
  int cap = 0;                // rows the activation buffers hold
  DBuf<float> Z1, Z2, Y, T, dY, dH2, dZ2, dH1, dZ1;
  DBuf<bf16> Xb, H1b, H2b, dYb, dZ2b, dZ1b;
  DBuf<double> part;
  DBuf<int> idx;
};

namespace {

int ensure_cap(ci_mlp* M, int rows) {
  if (rows <= M->cap) return CI_OK;
  const size_t r = rows;
  CM_CUDA(M->Z1.alloc(r * M->H));
  CM_CUDA(M->Z2.alloc(r * M->H));
  CM_CUDA(M->Y.alloc(r * M->n_out));
  CM_CUDA(M->T.alloc(r * M->n_out));
  CM_CUDA(M->dY.alloc(r * M->n_out));
  CM_CUDA(M->dH2.alloc(r * M->H));
  CM_CUDA(M->dZ2.alloc(r * M->H));
  CM_CUDA(M->dH1.alloc(r * M->H));
  CM_CUDA(M->dZ1.alloc(r * M->H));
  CM_CUDA(M->Xb.alloc(r * M->n_in));
  CM_CUDA(M->H1b.alloc(r * M->H));
  CM_CUDA(M->H2b.alloc(r * M->H));
  CM_CUDA(M->dYb.alloc(r * M->n_out));
  CM_CUDA(M->dZ2b.alloc(r * M->H));
  CM_CUDA(M->dZ1b.alloc(r * M->H));
  CM_CUDA(M->part.alloc(nb(r * M->n_out)));
  CM_CUDA(M->idx.alloc(r));
  M->cap = rows;
  return CI_OK;
}

int gemm(ci_mlp* M, const void* A, int lda, int tA, const void* B, int ldb, int tB, float* C, int ldc,
         void* Cb, int m, int n, int k, float beta, const float* bias, int act, cudaStream_t st) {
  return ci_gemm_bf16(A, lda, tA, B, ldb, tB, C, ldc, Cb, m, n, k, 1.0f, beta, bias, act,
                      M->err.p, st);
}

// forward of `rows` rows already in Xb; writes Y (and the hidden activations)
int forward(ci_mlp* M, int rows, cudaStream_t st) {
  const bf16* W1 = M->pb.p + M->off[0];
  const bf16* W2 = M->pb.p + M->off[2];
  const bf16* W3 = M->pb.p + M->off[4];
  const float* b1 = M->p.p + M->off[1];
  const float* b2 = M->p.p + M->off[3];
  const float* b3 = M->p.p + M->off[5];
  CM_OK(gemm(M, M->Xb.p, M->n_in, 0, W1, M->H, 0, M->Z1.p, M->H, M->H1b.p, rows, M->H, M->n_in, 0.f,
             b1, 1, st));
  CM_OK(gemm(M, M->H1b.p, M->H, 0, W2, M->H, 0, M->Z2.p, M->H, M->H2b.p, rows, M->H, M->H, 0.f, b2, 1,
             st));
  CM_OK(gemm(M, M->H2b.p, M->H, 0, W3, M->n_out, 0, M->Y.p, M->n_out, nullptr, rows, M->n_out, M->H,
             0.f, b3, 0, st));
  return CI_OK;
}

// loss and gradients into M->g for `rows` rows in Xb / T; *loss (may be NULL) gets the
// mean squared error (host, synchronises)
int backward(ci_mlp* M, int rows, cudaStream_t st, double* loss) {
  const long long ny = (long long)rows * M->n_out, nh = (long long)rows * M->H;
  k_mse_grad<<<nb(ny), 256, 0, st>>>(M->Y.p, M->T.p, M->dY.p, M->dYb.p, ny, 2.0f / (float)ny,
                                     M->part.p);
  float* gW1 = M->g.p + M->off[0];
  float* gb1 = M->g.p + M->off[1];
  float* gW2 = M->g.p + M->off[2];
  float* gb2 = M->g.p + M->off[3];
  float* gW3 = M->g.p + M->off[4];
  float* gb3 = M->g.p + M->off[5];
  const bf16* W2 = M->pb.p + M->off[2];
  const bf16* W3 = M->pb.p + M->off[4];
  // layer 3
  CM_OK(gemm(M, M->H2b.p, M->H, 1, M->dYb.p, M->n_out, 0, gW3, M->n_out, nullptr, M->H, M->n_out,
             rows, 0.f, nullptr, 0, st));
  k_colsum<<<nb(M->n_out), 256, 0, st>>>(M->dY.p, rows, M->n_out, gb3);
  CM_OK(gemm(M, M->dYb.p, M->n_out, 0, W3, M->n_out, 1, M->dH2.p, M->H, nullptr, rows, M->H,
             M->n_out, 0.f, nullptr, 0, st));
  // Z2 holds tanh(Z2) = H2 (the GEMM wrote the activated values)
  k_tanh_back<<<nb(nh), 256, 0, st>>>(M->dH2.p, M->Z2.p, M->dZ2.p, M->dZ2b.p, nh);
  // layer 2
  CM_OK(gemm(M, M->H1b.p, M->H, 1, M->dZ2b.p, M->H, 0, gW2, M->H, nullptr, M->H, M->H, rows, 0.f,
             nullptr, 0, st));
  k_colsum<<<nb(M->H), 256, 0, st>>>(M->dZ2.p, rows, M->H, gb2);
  CM_OK(gemm(M, M->dZ2b.p, M->H, 0, W2, M->H, 1, M->dH1.p, M->H, nullptr, rows, M->H, M->H, 0.f,
             nullptr, 0, st));
  k_tanh_back<<<nb(nh), 256, 0, st>>>(M->dH1.p, M->Z1.p, M->dZ1.p, M->dZ1b.p, nh);
  // layer 1
  CM_OK(gemm(M, M->Xb.p, M->n_in, 1, M->dZ1b.p, M->H, 0, gW1, M->H, nullptr, M->n_in, M->H, rows,
             0.f, nullptr, 0, st));
  k_colsum<<<nb(M->H), 256, 0, st>>>(M->dZ1.p, rows, M->H, gb1);
  CM_CUDA(cudaGetLastError());
  if (loss) {
    std::vector<double> part(nb(ny));
    CM_CUDA(cudaMemcpyAsync(part.data(), M->part.p, sizeof(double) * part.size(),
                            cudaMemcpyDeviceToHost, st));
    CM_CUDA(cudaStreamSynchronize(st));
    double s = 0.0;
    for (double x : part) s += x;
    *loss = s / (double)ny;
  }
  return CI_OK;
}

int check_err(ci_mlp* M, cudaStream_t st) {
  int e = 0;
  CM_CUDA(cudaMemcpyAsync(&e, M->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CM_CUDA(cudaStreamSynchronize(st));
  if (e) return ci::set_last_error(CI_ERR_CUDA, "tensor-core GEMM wait timed out");
  return CI_OK;
}

}  // namespace

extern "C" {

int ci_mlp_create(int n_in, int n_hidden, int n_out, unsigned long long seed, ci_mlp** out) {
  if (!out || n_in <= 0 || n_hidden <= 0 || n_out <= 0)
    return ci::set_last_error(CI_ERR_INVALID, "ci_mlp_create: bad sizes");
  ci_mlp* M = new ci_mlp();
  M->n_in = n_in;
  M->H = n_hidden;
  M->n_out = n_out;
  const long long sz[6] = {(long long)n_in * n_hidden, n_hidden, (long long)n_hidden * n_hidden,
                           n_hidden, (long long)n_hidden * n_out, n_out};
  long long o = 0;
  for (int i = 0; i < 6; i++) {
    M->off[i] = o;
    o += sz[i];
  }
  M->np = o;
  // Glorot-uniform weights, zero biases, from the seed
  std::vector<float> h(o, 0.f);
  std::mt19937_64 rng(seed);
  const int fan[3][2] = {{n_in, n_hidden}, {n_hidden, n_hidden}, {n_hidden, n_out}};
  for (int l = 0; l < 3; l++) {
    const double a = std::sqrt(6.0 / (fan[l][0] + fan[l][1]));
    std::uniform_real_distribution<double> U(-a, a);
    for (long long i = 0; i < sz[2 * l]; i++) h[M->off[2 * l] + i] = (float)U(rng);
  }
  int rc = CI_OK;
  if (M->p.alloc(o) || M->g.alloc(o) || M->m.alloc(o) || M->v.alloc(o) || M->pb.alloc(o) ||
      M->err.alloc(1))
    rc = ci::set_last_error(CI_ERR_NOMEM, "ci_mlp_create: device allocation failed");
  if (!rc) rc = ci_mlp_set_params(M, h.data());
  if (!rc && (cudaMemset(M->m.p, 0, sizeof(float) * o) || cudaMemset(M->v.p, 0, sizeof(float) * o) ||
              cudaMemset(M->err.p, 0, sizeof(int))))
    rc = ci::set_last_error(CI_ERR_CUDA, "ci_mlp_create: memset failed");
  if (rc) {
    delete M;
    return rc;
  }
  *out = M;
  return CI_OK;
}

int ci_mlp_destroy(ci_mlp* M) {
  delete M;
  return CI_OK;
}

long long ci_mlp_num_params(const ci_mlp* M) { return M ? M->np : 0; }

int ci_mlp_set_params(ci_mlp* M, const float* h) {
  if (!M || !h) return ci::set_last_error(CI_ERR_INVALID, "null argument");
  CM_CUDA(cudaMemcpy(M->p.p, h, sizeof(float) * M->np, cudaMemcpyHostToDevice));
  k_to_bf16<<<nb(M->np), 256>>>(M->p.p, M->pb.p, M->np);
  CM_CUDA(cudaGetLastError());
  CM_CUDA(cudaDeviceSynchronize());
  M->step = 0;
  return CI_OK;
}

int ci_mlp_get_params(ci_mlp* M, float* h) {
  if (!M || !h) return ci::set_last_error(CI_ERR_INVALID, "null argument");
  CM_CUDA(cudaMemcpy(h, M->p.p, sizeof(float) * M->np, cudaMemcpyDeviceToHost));
  return CI_OK;
}

int ci_mlp_predict(ci_mlp* M, const float* d_X, int n, float* d_Y, void* stream) {
  if (!M || !d_X || !d_Y || n <= 0) return ci::set_last_error(CI_ERR_INVALID, "bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (int r0 = 0; r0 < n; r0 += 4096) {
    const int rows = std::min(4096, n - r0);
    CM_OK(ensure_cap(M, rows));
    k_to_bf16<<<nb((long long)rows * M->n_in), 256, 0, st>>>(d_X + (size_t)r0 * M->n_in, M->Xb.p,
                                                             (long long)rows * M->n_in);
    CM_OK(forward(M, rows, st));
    CM_CUDA(cudaMemcpyAsync(d_Y + (size_t)r0 * M->n_out, M->Y.p, sizeof(float) * rows * M->n_out,
                            cudaMemcpyDeviceToDevice, st));
  }
  return check_err(M, st);
}

int ci_mlp_gradients(ci_mlp* M, const float* d_X, const float* d_T, int n, float* h_grad,
                     double* loss) {
  if (!M || !d_X || !d_T || n <= 0) return ci::set_last_error(CI_ERR_INVALID, "bad argument");
  CM_OK(ensure_cap(M, n));
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  CM_CUDA(cudaMemcpy(M->idx.p, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  k_gather_rows<<<n, 128>>>(d_X, d_T, M->idx.p, n, M->n_in, M->n_out, M->Xb.p, M->T.p);
  CM_OK(forward(M, n, 0));
  CM_OK(backward(M, n, 0, loss));
  if (h_grad) CM_CUDA(cudaMemcpy(h_grad, M->g.p, sizeof(float) * M->np, cudaMemcpyDeviceToHost));
  return check_err(M, 0);
}

int ci_mlp_train(ci_mlp* M, const float* d_X, const float* d_T, int n, int batch, int epochs,
                 float lr, unsigned long long seed, double* h_loss, void* stream) {
  if (!M || !d_X || !d_T || n <= 0 || batch <= 0 || epochs <= 0)
    return ci::set_last_error(CI_ERR_INVALID, "bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  batch = std::min(batch, n);
  CM_OK(ensure_cap(M, n));
  std::mt19937_64 rng(seed);
  std::vector<int> perm(n);
  for (int i = 0; i < n; i++) perm[i] = i;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ep++) {
    std::shuffle(perm.begin(), perm.end(), rng);
    CM_CUDA(cudaMemcpyAsync(M->idx.p, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    double ep_loss = 0.0;
    int nbatches = 0;
    for (int b0 = 0; b0 + batch <= n; b0 += batch) {
      k_gather_rows<<<batch, 128, 0, st>>>(d_X, d_T, M->idx.p + b0, batch, M->n_in, M->n_out,
                                           M->Xb.p, M->T.p);
      CM_OK(forward(M, batch, st));
      const bool last = b0 + 2 * batch > n;
      double l = 0.0;
      CM_OK(backward(M, batch, st, (h_loss && last) ? &l : nullptr));
      ep_loss += l;
      nbatches += last ? 1 : 0;
      M->step++;
      const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
      k_adam<<<nb(M->np), 256, 0, st>>>(M->p.p, M->g.p, M->m.p, M->v.p, M->pb.p, M->np, lr, b1, b2,
                                        eps, c1, c2);
      CM_CUDA(cudaGetLastError());
    }
    if (h_loss) h_loss[ep] = nbatches ? ep_loss / nbatches : 0.0;
  }
  return check_err(M, st);
}

}  // extern "C"
