// ci_noalloc.cu -- ci_strain_energy_noalloc: the strain-energy reduction of
// ci_strain_energy for callers that cannot allocate device memory.
//
// Who needs it: a host program that owns every byte of device memory (its own pool or
// arena sized at start-up) and forbids driver allocations afterwards, a plug-in
// embedded in such a program, or a time-critical loop in which cudaMalloc/cudaFree
// are unacceptable because they may synchronise the device or fail under memory
// pressure.  Those callers already hold their mesh, displacement and output buffers
// on the device; this entry point reads and writes only those, plus a fixed scratch
// array compiled into the library.
//
// The scratch is a file-scope __device__ array: every GPU that loads the library
// holds it (kMaxBlocks x 2 doubles = 256 KiB, plus one status word) until the
// process exits.  Host code cannot use the array's name as a device address (it is a
// host-side shadow), so the first call on each device looks up the real address with
// cudaGetSymbolAddress while that device is current, and passes it to the kernels.
// Do that first call outside any stream capture.  The cached addresses belong to the
// device's primary context: after cudaDeviceReset (or anything else that destroys that
// context) this entry point must not be called again in the same process.  All calls
// share the array and see what the previous call left there: every block rewrites its
// own partial sums, and the status word is cleared by the reduction that consumes it.
// Calls that overlap on the GPU (for example on two streams) race on the array and
// must be serialised by the caller.
//
// The connectivity is already on the device, so it cannot be validated on the host:
// an element with a node index outside [0, num_nodes) is skipped (no load of x or u
// through that index) and sets a status bit that turns both outputs into NaN.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/cppimpact_gb300.h"
#include "ci_kernels.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = CI_NOALLOC_MAX_ELEMENTS / kThreads;
constexpr int kMaxDevices = 64;
constexpr unsigned int kBadIndex = 4u;  // beside ci::ST_DEGENERATE (1) and ST_NONFINITE (2)

// per-block partial (energy, volume) of one call: block b writes entries 2b and 2b + 1
static __device__ __align__(256) double g_partials[2 * kMaxBlocks];
static __device__ __align__(256) unsigned int g_status;

std::mutex g_mu;
double* g_partials_ptr[kMaxDevices] = {};
unsigned int* g_status_ptr[kMaxDevices] = {};

// Element strain energy 1/2 eps:D:eps and volume, one thread per element, geometry
// relative to the element's first node so FP32 keeps the element's resolution.
template <int NPE>
__global__ void __launch_bounds__(kThreads) k_energy_partials(const double* __restrict__ x,
                                                              const int* __restrict__ conn,
                                                              const double* __restrict__ u, int N,
                                                              int E, ci::ElemParams p,
                                                              double* partials,
                                                              unsigned int* status) {
  __shared__ float red[kThreads / 32];
  const int e = blockIdx.x * kThreads + threadIdx.x;
  float wint = 0.f, wp = 0.f, vol = 0.f;
  int n[NPE];
  bool ok = e < E;
  if (ok) {
#pragma unroll
    for (int a = 0; a < NPE; a++) {
      n[a] = conn[(size_t)NPE * e + a];
      ok = ok && (unsigned)n[a] < (unsigned)N;
    }
    if (!ok) atomicOr(status, kBadIndex);
  }
  if (ok) {
    float xe[NPE][3], ue[NPE][3];
#pragma unroll
    for (int a = 0; a < NPE; a++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        xe[a][k] = (float)(x[3 * (size_t)n[a] + k] - x[3 * (size_t)n[0] + k]);
        ue[a][k] = (float)u[3 * (size_t)n[a] + k];
      }
    ci::DevState S{};
    S.status = status;
    float f[NPE][3];
    ci::element_force<NPE, ci::EM_REFCOMPAT>(p, S, e, E, xe, ue, f, wint, wp, vol);
  }
  const float t0 = ci::block_sum<kThreads>(wint, red);
  const float t1 = ci::block_sum<kThreads>(vol, red);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = (double)t0;
    partials[2 * blockIdx.x + 1] = (double)t1;
  }
}

// Fixed-order sum of the block partials; a degenerate element makes the energy NaN,
// an out-of-range node index both outputs.
__global__ void k_energy_reduce(const double* partials, int nblocks, unsigned int* status,
                                double* out) {
  __shared__ double red[2][kThreads];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += kThreads) {
    a += partials[2 * i];
    b += partials[2 * i + 1];
  }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const unsigned int st = *status;
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    out[0] = st ? nan : red[0][0];
    out[1] = (st & kBadIndex) ? nan : red[1][0];
    *status = 0u;
  }
}

}  // namespace

namespace ci {
int set_last_error(int code, const char* msg);  // ci_solver.cu
}

namespace {
int fail(int code, const char* msg) { return ci::set_last_error(code, msg); }
}  // namespace

extern "C" int ci_strain_energy_noalloc(const double* d_xloc, const int* d_element_nodes,
                                        int num_nodes, int num_elements, int nodes_per_element,
                                        const double* d_u, double E, double nu, double* d_out,
                                        void* stream) {
  if (!d_xloc || !d_element_nodes || !d_u || !d_out || num_nodes <= 0 || num_elements <= 0)
    return fail(CI_ERR_INVALID, "ci_strain_energy_noalloc: null pointer or empty mesh");
  if (nodes_per_element != 4 && nodes_per_element != 10)
    return fail(CI_ERR_UNSUPPORTED, "ci_strain_energy_noalloc: nodes_per_element must be 4 or 10");
  if (num_elements > CI_NOALLOC_MAX_ELEMENTS)
    return fail(CI_ERR_TOO_LARGE,
                "ci_strain_energy_noalloc: more than CI_NOALLOC_MAX_ELEMENTS elements");
  if (!(E > 0.0) || !(nu > -1.0 && nu < 0.5))
    return fail(CI_ERR_INVALID, "ci_strain_energy_noalloc: needs E > 0 and -1 < nu < 0.5");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(CI_ERR_CUDA, "ci_strain_energy_noalloc: no usable current device");
  double* partials;
  unsigned int* status;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_partials_ptr[dev]) {
      // once per device, with that device current: the device addresses of the arrays
      void* pp = nullptr;
      void* ps = nullptr;
      if (cudaGetSymbolAddress(&pp, g_partials) != cudaSuccess ||
          cudaGetSymbolAddress(&ps, g_status) != cudaSuccess)
        return fail(CI_ERR_CUDA, "ci_strain_energy_noalloc: cudaGetSymbolAddress failed");
      g_partials_ptr[dev] = static_cast<double*>(pp);
      g_status_ptr[dev] = static_cast<unsigned int*>(ps);
    }
    partials = g_partials_ptr[dev];
    status = g_status_ptr[dev];
  }
  ci::ElemParams p{};
  p.dt = 1.0f;
  p.mu = (float)(E / (2.0 * (1.0 + nu)));
  p.lambda = (float)(E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
  p.accum_energy = 1;
  const int nb = (num_elements + kThreads - 1) / kThreads;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (nodes_per_element == 4)
    k_energy_partials<4><<<nb, kThreads, 0, st>>>(d_xloc, d_element_nodes, d_u, num_nodes,
                                                  num_elements, p, partials, status);
  else
    k_energy_partials<10><<<nb, kThreads, 0, st>>>(d_xloc, d_element_nodes, d_u, num_nodes,
                                                   num_elements, p, partials, status);
  k_energy_reduce<<<1, kThreads, 0, st>>>(partials, nb, status, d_out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CI_ERR_CUDA, cudaGetErrorString(e));
  return CI_OK;
}
