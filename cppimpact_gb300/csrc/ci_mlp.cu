// ci_mlp.cu -- the surrogate's MLP (n_in -> H -> H -> n_out, tanh hidden layers):
// forward, backward and Adam on the GPU, every matrix product through ci_gemm_bf16
// (BF16 operands, FP32 accumulation), FP32 master weights, fixed-order reductions.
// The products of layers 2 and 3 are arranged as A B^T with both operands K-major (the
// form of the TMA-pipelined tcgen05 kernel): BF16 copies of W2 and W3 are kept
// transposed, and the weight gradients read transposed activations and output
// gradients.
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

// dY = scale (Y - T) (scale = 2 / (rows * cols)) for row r = blockIdx.y, whose targets
// are row idx[r] of T (row r when idx is null); with LOSS, per-block partial sums of
// (Y - T)^2
template <bool LOSS>
__global__ void k_mse_grad(const float* Y, const float* T, const int* idx, int cols, float* dY,
                           bf16* dYb, float scale, double* part) {
  __shared__ double red[256];
  const int r = blockIdx.y, c = blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (c < cols) {
    const size_t i = (size_t)r * cols + c;
    const float d = Y[i] - T[(size_t)(idx ? idx[r] : r) * cols + c];
    dY[i] = scale * d;
    dYb[i] = __float2bfloat16(scale * d);
    s = (double)d * d;
  }
  if (!LOSS) return;
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
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

// column sums of a [rows x cols] matrix: 32 columns per CTA, 8 row groups (rows
// r = g, g + 8, ... in order), then the 8 partial sums in group order
__global__ void __launch_bounds__(256) k_colsum(const float* A, int rows, int cols, float* out) {
  __shared__ float part[8][33];
  const int tx = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + tx;
  float s = 0.f;
  if (c < cols)
    for (int r = g; r < rows; r += 8) s += A[(size_t)r * cols + c];
  part[g][tx] = s;
  __syncthreads();
  if (g == 0 && c < cols) {
    float t = part[0][tx];
    for (int k = 1; k < 8; k++) t += part[k][tx];
    out[c] = t;
  }
}

// Layer 1 when n_in is small (the surrogate's 4 impact parameters): Z = tanh(X W1 + b1)
// with the BF16 operands of the GEMM path, FP32 products summed in input order; writes
// the FP32 activation and its BF16 copy.
__global__ void k_layer1_fwd(const bf16* X, const bf16* W1, const float* b1, int rows, int n_in,
                             int H, float* Z, bf16* Hb) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)rows * H) return;
  const int r = (int)(i / H), h = (int)(i % H);
  float acc = 0.f;
  for (int k = 0; k < n_in; k++)
    acc = fmaf(__bfloat162float(X[(size_t)r * n_in + k]), __bfloat162float(W1[(size_t)k * H + h]), acc);
  const float z = tanhf(acc + b1[h]);
  Z[i] = z;
  Hb[i] = __float2bfloat16(z);
}

// gW1 = X^T dZ1 [n_in x H] for small n_in: one warp per entry; lane j sums rows j, j+32,
// ... in order, then the 32 lane sums in a fixed butterfly order
__global__ void k_layer1_wgrad(const bf16* X, const bf16* dZb, int rows, int n_in, int H, float* gW) {
  const int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= n_in * H) return;
  const int k = w / H, h = w % H;
  float acc = 0.f;
  for (int r = lane; r < rows; r += 32)
    acc = fmaf(__bfloat162float(X[(size_t)r * n_in + k]), __bfloat162float(dZb[(size_t)r * H + h]), acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) gW[w] = acc;
}

// out [cols x rows] (leading dimension ld_out) = in^T, in [rows x cols] (ld_in); 32 x 32
// tiles through shared memory
__global__ void __launch_bounds__(256) k_transpose_bf16(const bf16* in, int rows, int cols,
                                                        int ld_in, bf16* out, int ld_out) {
  __shared__ bf16 tile[32][34];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int k = ty; k < 32; k += 8) {
    const int r = r0 + k, c = c0 + tx;
    if (r < rows && c < cols) tile[k][tx] = in[(size_t)r * ld_in + c];
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int c = c0 + k, r = r0 + tx;
    if (r < rows && c < cols) out[(size_t)c * ld_out + r] = tile[tx][k];
  }
}

inline cudaError_t transpose_bf16(const bf16* in, int rows, int cols, bf16* out, cudaStream_t st) {
  const dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_bf16<<<grid, 256, 0, st>>>(in, rows, cols, cols, out, rows);
  return cudaGetLastError();
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

// rows of X picked by idx -> Xb (BF16)
__global__ void k_gather_rows(const float* X, const int* idx, int rows, int nx, bf16* Xb) {
  const int r = blockIdx.x;
  if (r >= rows) return;
  const int s = idx[r];
  for (int j = threadIdx.x; j < nx; j += blockDim.x)
    Xb[(size_t)r * nx + j] = __float2bfloat16(X[(size_t)s * nx + j]);
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
  DBuf<bf16> wT;              // BF16 W2^T [H x H] then W3^T [n_out x H]
  DBuf<int> err;
  long long step = 0;
  int cap = 0;                // rows the activation buffers hold
  DBuf<float> Z1, Z2, Y, dY, dH2, dZ2, dH1, dZ1;
  DBuf<bf16> Xb, H1b, H2b, dYb, dZ2b, dZ1b;
  DBuf<bf16> H1bT, H2bT, dYbT, dZ2bT;  // transposes [cols x rows] for the weight gradients
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
  CM_CUDA(M->H1bT.alloc(r * M->H));
  CM_CUDA(M->H2bT.alloc(r * M->H));
  CM_CUDA(M->dYbT.alloc(r * M->n_out));
  CM_CUDA(M->dZ2bT.alloc(r * M->H));
  CM_CUDA(M->part.alloc(r * nb(M->n_out)));
  CM_CUDA(M->idx.alloc(r));
  M->cap = rows;
  return CI_OK;
}

int gemm(ci_mlp* M, const void* A, int lda, int tA, const void* B, int ldb, int tB, float* C, int ldc,
         void* Cb, int m, int n, int k, float beta, const float* bias, int act, cudaStream_t st) {
  return ci_gemm_bf16(A, lda, tA, B, ldb, tB, C, ldc, Cb, m, n, k, 1.0f, beta, bias, act,
                      M->err.p, st);
}

// BF16 W2^T and W3^T from the BF16 parameter copy (after every parameter update)
int refresh_wT(ci_mlp* M, cudaStream_t st) {
  CM_CUDA(transpose_bf16(M->pb.p + M->off[2], M->H, M->H, M->wT.p, st));
  CM_CUDA(transpose_bf16(M->pb.p + M->off[4], M->H, M->n_out, M->wT.p + (size_t)M->H * M->H, st));
  return CI_OK;
}

// forward of `rows` rows already in Xb; writes Y (and the hidden activations)
int forward(ci_mlp* M, int rows, cudaStream_t st) {
  const bf16* W1 = M->pb.p + M->off[0];
  const bf16* W2T = M->wT.p;
  const bf16* W3T = M->wT.p + (size_t)M->H * M->H;
  const float* b1 = M->p.p + M->off[1];
  const float* b2 = M->p.p + M->off[3];
  const float* b3 = M->p.p + M->off[5];
  if (M->n_in < 16) {
    k_layer1_fwd<<<nb((long long)rows * M->H), 256, 0, st>>>(M->Xb.p, W1, b1, rows, M->n_in, M->H,
                                                             M->Z1.p, M->H1b.p);
    CM_CUDA(cudaGetLastError());
  } else {
    CM_OK(gemm(M, M->Xb.p, M->n_in, 0, W1, M->H, 0, M->Z1.p, M->H, M->H1b.p, rows, M->H, M->n_in,
               0.f, b1, 1, st));
  }
  CM_OK(gemm(M, M->H1b.p, M->H, 0, W2T, M->H, 1, M->Z2.p, M->H, M->H2b.p, rows, M->H, M->H, 0.f, b2,
             1, st));
  CM_OK(gemm(M, M->H2b.p, M->H, 0, W3T, M->H, 1, M->Y.p, M->n_out, nullptr, rows, M->n_out, M->H,
             0.f, b3, 0, st));
  return CI_OK;
}

// loss and gradients into M->g for `rows` rows in Xb, whose targets are rows idx[r] of T
// (rows r when idx is null); *loss (may be NULL) gets the mean squared error (host,
// synchronises)
int backward(ci_mlp* M, int rows, cudaStream_t st, double* loss, const float* T, const int* idx) {
  const long long ny = (long long)rows * M->n_out, nh = (long long)rows * M->H;
  const dim3 mse_grid(nb(M->n_out), rows);
  if (loss)
    k_mse_grad<true><<<mse_grid, 256, 0, st>>>(M->Y.p, T, idx, M->n_out, M->dY.p, M->dYb.p,
                                               2.0f / (float)ny, M->part.p);
  else
    k_mse_grad<false><<<mse_grid, 256, 0, st>>>(M->Y.p, T, idx, M->n_out, M->dY.p, M->dYb.p,
                                                2.0f / (float)ny, M->part.p);
  float* gW1 = M->g.p + M->off[0];
  float* gb1 = M->g.p + M->off[1];
  float* gW2 = M->g.p + M->off[2];
  float* gb2 = M->g.p + M->off[3];
  float* gW3 = M->g.p + M->off[4];
  float* gb3 = M->g.p + M->off[5];
  const bf16* W2 = M->pb.p + M->off[2];
  const bf16* W3 = M->pb.p + M->off[4];
  // layer 3: gW3 = H2^T dY as (H2^T) (dY^T)^T
  CM_CUDA(transpose_bf16(M->H2b.p, rows, M->H, M->H2bT.p, st));
  CM_CUDA(transpose_bf16(M->dYb.p, rows, M->n_out, M->dYbT.p, st));
  CM_OK(gemm(M, M->H2bT.p, rows, 0, M->dYbT.p, rows, 1, gW3, M->n_out, nullptr, M->H, M->n_out,
             rows, 0.f, nullptr, 0, st));
  k_colsum<<<(M->n_out + 31) / 32, 256, 0, st>>>(M->dY.p, rows, M->n_out, gb3);
  CM_OK(gemm(M, M->dYb.p, M->n_out, 0, W3, M->n_out, 1, M->dH2.p, M->H, nullptr, rows, M->H,
             M->n_out, 0.f, nullptr, 0, st));
  // Z2 holds tanh(Z2) = H2 (the GEMM wrote the activated values)
  k_tanh_back<<<nb(nh), 256, 0, st>>>(M->dH2.p, M->Z2.p, M->dZ2.p, M->dZ2b.p, nh);
  // layer 2: gW2 = H1^T dZ2 as (H1^T) (dZ2^T)^T
  CM_CUDA(transpose_bf16(M->H1b.p, rows, M->H, M->H1bT.p, st));
  CM_CUDA(transpose_bf16(M->dZ2b.p, rows, M->H, M->dZ2bT.p, st));
  CM_OK(gemm(M, M->H1bT.p, rows, 0, M->dZ2bT.p, rows, 1, gW2, M->H, nullptr, M->H, M->H, rows, 0.f,
             nullptr, 0, st));
  k_colsum<<<(M->H + 31) / 32, 256, 0, st>>>(M->dZ2.p, rows, M->H, gb2);
  CM_OK(gemm(M, M->dZ2b.p, M->H, 0, W2, M->H, 1, M->dH1.p, M->H, nullptr, rows, M->H, M->H, 0.f,
             nullptr, 0, st));
  k_tanh_back<<<nb(nh), 256, 0, st>>>(M->dH1.p, M->Z1.p, M->dZ1.p, M->dZ1b.p, nh);
  // layer 1
  if (M->n_in < 16) {
    k_layer1_wgrad<<<nb(32LL * M->n_in * M->H), 256, 0, st>>>(M->Xb.p, M->dZ1b.p, rows, M->n_in,
                                                               M->H, gW1);
    CM_CUDA(cudaGetLastError());
  } else {
    CM_OK(gemm(M, M->Xb.p, M->n_in, 1, M->dZ1b.p, M->H, 0, gW1, M->H, nullptr, M->n_in, M->H, rows,
               0.f, nullptr, 0, st));
  }
  k_colsum<<<(M->H + 31) / 32, 256, 0, st>>>(M->dZ1.p, rows, M->H, gb1);
  CM_CUDA(cudaGetLastError());
  if (loss) {
    std::vector<double> part((size_t)rows * nb(M->n_out));
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
      M->wT.alloc((size_t)n_hidden * n_hidden + (size_t)n_hidden * n_out) || M->err.alloc(1))
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
  CM_OK(refresh_wT(M, 0));
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
  k_gather_rows<<<n, 32>>>(d_X, M->idx.p, n, M->n_in, M->Xb.p);
  CM_OK(forward(M, n, 0));
  CM_OK(backward(M, n, 0, loss, d_T, nullptr));
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
      k_gather_rows<<<batch, 32, 0, st>>>(d_X, M->idx.p + b0, batch, M->n_in, M->Xb.p);
      CM_OK(forward(M, batch, st));
      const bool last = b0 + 2 * batch > n;
      double l = 0.0;
      CM_OK(backward(M, batch, st, (h_loss && last) ? &l : nullptr, d_T, M->idx.p + b0));
      ep_loss += l;
      nbatches += last ? 1 : 0;
      M->step++;
      const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
      k_adam<<<nb(M->np), 256, 0, st>>>(M->p.p, M->g.p, M->m.p, M->v.p, M->pb.p, M->np, lr, b1, b2,
                                        eps, c1, c2);
      CM_CUDA(cudaGetLastError());
      CM_OK(refresh_wT(M, st));
    }
    if (h_loss) h_loss[ep] = nbatches ? ep_loss / nbatches : 0.0;
  }
  return check_err(M, st);
}

}  // extern "C"
