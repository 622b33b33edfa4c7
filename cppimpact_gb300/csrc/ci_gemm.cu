// ci_gemm.cu -- BF16 tensor-core GEMM on sm_103a (tcgen05 + TMEM), FP32 accumulation.
//
//   C[M x N] (+)= alpha * op(A)[M x K] * op(B)[K x N]  (+ bias[N]) (then optional tanh)
//
// A, B are BF16 in global memory, row-major with leading dimensions lda/ldb; op() is a
// transpose flag per operand.  C is FP32 (row-major, ldc); an optional BF16 copy of C
// is written for the next layer.  This is the dense contraction of the surrogate (POD
// projections and the MLP's forward/backward passes); the impact step itself has none.
//
// One CTA computes a 128 x BN tile (BN = 64 or 128).  Per K-tile of 64:
//  1. all 128 threads stage A (128 x 64) and B (BN x 64) as K-major BF16 in shared
//     memory, in the canonical no-swizzle layout of 8-row x 16-byte core matrices
//     (core matrix (r/8, k/8) at r/8 * SBO + k/8 * LBO, LBO = 128 B, SBO = 1024 B);
//  2. fence.proxy.async makes the writes visible to the tensor core; one elected
//     thread issues 4 x tcgen05.mma.kind::f16 (K = 16 each) into the TMEM accumulator
//     and commits to an mbarrier;
//  3. every thread waits on the mbarrier (bounded spin: on timeout the kernel records
//     an error flag, frees its TMEM and returns) before the stage is overwritten.
// The epilogue reads the accumulator with tcgen05.ld (each warp its 32 TMEM lanes =
// 32 rows), applies alpha, beta, bias, tanh and stores.
//
// C = A B^T with both operands K-major (transA = 0, transB = 1), M >= 128 and aligned
// rows takes a pipelined kernel instead: TMA (cp.async.bulk.tensor, 128-byte swizzle)
// streams 128 x 64 and BN x 64 tiles through a 4-stage shared-memory ring, one thread
// issues the TMA loads, one thread the MMAs, and mbarriers hand stages back and forth
// (full: TMA bytes landed; empty: the MMAs reading a stage completed).  Without split-K
// that kernel is persistent (k_gemm_tma_pers: one CTA per SM walking the tiles, two
// TMEM accumulators so the epilogue of one tile overlaps the MMAs of the next); with
// split-K (few output tiles, long K) it runs one CTA per (tile, K range).
#include <cuda.h>  // CUtensorMap and its enums; the encoder is fetched at run time
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>

#include "../../include/cppimpact_gb300.h"

namespace ci {
int set_last_error(int code, const char* msg);
}

namespace {

constexpr int BM = 128;
constexpr int BK = 64;
constexpr unsigned kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: start address, leading / stride byte
// offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // version
  return d;                // base offset 0, lbo mode 0, layout 0 (no swizzle)
}

// Instruction descriptor of tcgen05.mma.kind::f16: D FP32, A and B BF16, both K-major,
// N >> 3 and M >> 4.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4)      // D format F32
         | (1u << 7)    // A format BF16
         | (1u << 10)   // B format BF16
         | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  for (unsigned it = 0; it < kSpinLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// byte offset of element (r, k) of a K-major no-swizzle tile (LBO 128, SBO 1024)
__device__ __forceinline__ uint32_t kmajor_off(int r, int k) {
  return (uint32_t)((r >> 3) * 1024 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

template <int BN>
__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16* __restrict__ A, int lda,
                                                   int transA, const __nv_bfloat16* __restrict__ B,
                                                   int ldb, int transB, float* C, int ldc,
                                                   __nv_bfloat16* Cb, int M, int N, int K,
                                                   float alpha, float beta,
                                                   const float* __restrict__ bias, int act,
                                                   int* err, int k_chunk, float* partial) {
  __shared__ __align__(1024) uint8_t sA[BM * BK * 2];
  __shared__ __align__(1024) uint8_t sB[BN * BK * 2];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  // split-K: this CTA reduces K range [kb, ke); partial results go to partial[z]
  const int kb = blockIdx.z * k_chunk;
  const int ke = min(K, kb + k_chunk);

  if (warp == 0) {
    // TMEM: BN columns (power of two >= 32) for the 128 x BN FP32 accumulator
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = instr_desc(BM, BN);
  bool ok = true;
  uint32_t phase = 0;
  const int ktiles = (ke - kb + BK - 1) / BK;
  for (int kt = 0; kt < ktiles && ok; kt++) {
    const int k0 = kb + kt * BK;
    // stage A: 128 rows x 64 k; consecutive threads read consecutive addresses
    for (int i = tid; i < BM * BK; i += 128) {
      const int r = transA ? i % BM : i / BK, k = transA ? i / BM : i % BK;
      const int gm = m0 + r, gk = k0 + k;
      __nv_bfloat16 v = __float2bfloat16(0.f);
      if (gm < M && gk < ke) v = transA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      *reinterpret_cast<__nv_bfloat16*>(sA + kmajor_off(r, k)) = v;
    }
    // stage B as K-major rows n: B_op[k][n]
    for (int i = tid; i < BN * BK; i += 128) {
      const int n = transB ? i / BK : i % BN, k = transB ? i % BK : i / BN;
      const int gn = n0 + n, gk = k0 + k;
      __nv_bfloat16 v = __float2bfloat16(0.f);
      if (gn < N && gk < ke) v = transB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
      *reinterpret_cast<__nv_bfloat16*>(sB + kmajor_off(n, k)) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < BK / 16; kk++) {
        // K = 16 per MMA = two core matrices along K = 2 x LBO bytes
        const uint64_t da = smem_desc(smem_u32(sA) + kk * 256, 128, 1024);
        const uint64_t db = smem_desc(smem_u32(sB) + kk * 256, 128, 1024);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              smem_u32(&bar))
          : "memory");
    }
    // CTA-uniform outcome: every thread leaves the loop at the same tile
    ok = __syncthreads_and(mbar_wait(smem_u32(&bar), phase)) != 0;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  }
  if (!ok) {
    // give the MMAs in flight one more bounded wait before the TMEM is freed
    mbar_wait(smem_u32(&bar), phase ^ 1u);
    if (tid == 0) atomicExch(err, 1);
  } else {
    // epilogue: warp w holds TMEM lanes [32w, 32w+32) = tile rows; 8 columns per load
    const int row = m0 + warp * 32 + lane;
    for (int c = 0; c < BN; c += 8) {
      uint32_t r[8];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < M && partial) {
        float* pr = partial + ((size_t)blockIdx.z * M + row) * N;
#pragma unroll
        for (int j = 0; j < 8; j++)
          if (n0 + c + j < N) pr[n0 + c + j] = ktiles > 0 ? __uint_as_float(r[j]) : 0.f;
      } else if (row < M) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int col = n0 + c + j;
          if (col >= N) continue;
          float v = alpha * __uint_as_float(r[j]);
          if (beta != 0.f) v += beta * C[(size_t)row * ldc + col];
          if (bias) v += bias[col];
          if (act == 1) v = tanhf(v);
          C[(size_t)row * ldc + col] = v;
          if (Cb) Cb[(size_t)row * ldc + col] = __float2bfloat16(v);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN)
                 : "memory");
}

constexpr int TBK = 64;      // K per stage: 64 BF16 = one 128-byte swizzle row
constexpr int TSTAGES = 4;

// Shared-memory descriptor of a K-major tile in the 128-byte swizzled layout TMA writes
// (rows of 128 bytes, 8-row groups 1024 bytes apart); LBO is unused for this layout.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;            // LBO (ignored) = 16 B
  d |= (uint64_t)(1024 >> 4) << 32;  // SBO: 8 rows x 128 B
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

template <int BN>
__global__ void __launch_bounds__(128, 1)
    k_gemm_tma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               float* C, int ldc, __nv_bfloat16* Cb, int M, int N, int K, float alpha, float beta,
               const float* __restrict__ bias, int act, int* err, int k_chunk, float* partial) {
  constexpr int A_BYTES = BM * TBK * 2;
  constexpr int B_BYTES = BN * TBK * 2;
  extern __shared__ uint8_t smem_raw[];
  // the swizzled tiles want 1024-byte alignment (the launch reserves the slack)
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + TSTAGES * A_BYTES;
  __shared__ __align__(8) uint64_t full[TSTAGES], empty[TSTAGES], done;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kb = blockIdx.z * k_chunk;
  const int ke = min(K, kb + k_chunk);
  const int ktiles = (ke - kb + TBK - 1) / TBK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < TSTAGES; s++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&done)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  bool ok = true;
  int issued = 0;
  if (warp == 0 && lane == 0) {
    // producer: stage kt waits until the MMAs of stage kt - TSTAGES released its slot
    for (int kt = 0; kt < ktiles; kt++) {
      const int s = kt % TSTAGES;
      if (kt >= TSTAGES && !mbar_wait(smem_u32(&empty[s]), ((kt / TSTAGES) - 1) & 1)) {
        ok = false;
        break;
      }
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                       smem_u32(&full[s])),
                   "r"(A_BYTES + B_BYTES)
                   : "memory");
      tma_load_2d(smem_u32(sA + s * A_BYTES), &tmA, kb + kt * TBK, m0, smem_u32(&full[s]));
      tma_load_2d(smem_u32(sB + s * B_BYTES), &tmB, kb + kt * TBK, n0, smem_u32(&full[s]));
      issued = kt + 1;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: 4 x (K = 16) per stage, accumulate in TMEM, release the stage
    const uint32_t idesc = instr_desc(BM, BN);
    for (int kt = 0; kt < ktiles; kt++) {
      const int s = kt % TSTAGES;
      if (!mbar_wait(smem_u32(&full[s]), (kt / TSTAGES) & 1)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < TBK / 16; kk++) {
        const uint64_t da = desc_sw128(smem_u32(sA + s * A_BYTES) + kk * 32);
        const uint64_t db = desc_sw128(smem_u32(sB + s * B_BYTES) + kk * 32);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              smem_u32(&empty[s]))
          : "memory");
    }
    // arrives once every MMA issued above has completed
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_u32(&done))
        : "memory");
  }
  const bool got = mbar_wait(smem_u32(&done), 0);
  ok = __syncthreads_and(ok && got) != 0;
  if (!ok) {
    // let the TMA loads still in flight land before the shared memory goes away
    if (warp == 0 && lane == 0)
      for (int kt = max(0, issued - TSTAGES); kt < issued; kt++)
        mbar_wait(smem_u32(&full[kt % TSTAGES]), (kt / TSTAGES) & 1);
    if (tid == 0) atomicExch(err, 1);
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const int row = m0 + warp * 32 + lane;
    for (int c = 0; c < BN; c += 8) {
      uint32_t r[8];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < M && partial) {
        float* pr = partial + ((size_t)blockIdx.z * M + row) * N + n0 + c;
        if (n0 + c + 8 <= N && (reinterpret_cast<uintptr_t>(pr) & 15) == 0 && ktiles > 0) {
          reinterpret_cast<float4*>(pr)[0] = make_float4(__uint_as_float(r[0]), __uint_as_float(r[1]),
                                                         __uint_as_float(r[2]), __uint_as_float(r[3]));
          reinterpret_cast<float4*>(pr)[1] = make_float4(__uint_as_float(r[4]), __uint_as_float(r[5]),
                                                         __uint_as_float(r[6]), __uint_as_float(r[7]));
        } else {
#pragma unroll
          for (int j = 0; j < 8; j++)
            if (n0 + c + j < N) pr[j] = ktiles > 0 ? __uint_as_float(r[j]) : 0.f;
        }
      } else if (row < M) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int col = n0 + c + j;
          v[j] = alpha * (ktiles > 0 ? __uint_as_float(r[j]) : 0.f);
          if (col < N) {
            if (beta != 0.f) v[j] += beta * C[(size_t)row * ldc + col];
            if (bias) v[j] += bias[col];
            if (act == 1) v[j] = tanhf(v[j]);
          }
        }
        float* crow = C + (size_t)row * ldc + n0 + c;
        if (n0 + c + 8 <= N && (reinterpret_cast<uintptr_t>(crow) & 15) == 0) {
          // this thread's 8 columns of its row as two 16-byte stores
          reinterpret_cast<float4*>(crow)[0] = make_float4(v[0], v[1], v[2], v[3]);
          reinterpret_cast<float4*>(crow)[1] = make_float4(v[4], v[5], v[6], v[7]);
        } else {
#pragma unroll
          for (int j = 0; j < 8; j++)
            if (n0 + c + j < N) crow[j] = v[j];
        }
        if (Cb)
#pragma unroll
          for (int j = 0; j < 8; j++)
            if (n0 + c + j < N) Cb[(size_t)row * ldc + n0 + c + j] = __float2bfloat16(v[j]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN)
                 : "memory");
}

// ---------------------------------------------------------------------------
// Persistent form of the A B^T kernel: one CTA per SM walks the output tiles (grouped
// raster: GM consecutive 128-row tiles share every BN-column tile, so the operand
// panels in flight stay in L2).  Six warps with fixed roles:
//   warp 0  TMA producer: 128 x 64 and BN x 64 tiles into a TSTAGES-deep ring;
//   warp 1  MMA issuer: tcgen05.mma into one of two TMEM accumulators (2 x BN columns),
//           tcgen05.commit releases ring stages and, after a tile's last K step,
//           hands the accumulator to the epilogue;
//   warps 2-5  epilogue: TMEM lane quarter (warp % 4), tcgen05.ld, alpha / beta / bias /
//           tanh, stores; then the accumulator goes back to the MMA issuer.
// The epilogue of tile i overlaps the MMAs of tile i + 1.  Every wait is bounded; a role
// that times out raises a shared abort flag so the others stop waiting, and the kernel
// reports the error through *err.
constexpr int PERS_THREADS = 192;
constexpr int GROUP_M = 16;

__device__ __forceinline__ bool mbar_wait_abort(uint32_t bar, uint32_t phase, volatile int* abort) {
  for (unsigned it = 0; it < kSpinLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
    if ((it & 255u) == 255u && *abort) return false;
  }
  *abort = 1;
  return false;
}

__device__ __forceinline__ void tile_coords(int t, int tiles_m, int tiles_n, int& mt, int& nt) {
  const int per_group = GROUP_M * tiles_n;
  const int g = t / per_group;
  const int m_base = g * GROUP_M;
  const int gm = min(GROUP_M, tiles_m - m_base);
  const int r = t - g * per_group;
  mt = m_base + r % gm;
  nt = r / gm;
}

template <int BN>
__global__ void __launch_bounds__(PERS_THREADS, 1)
    k_gemm_tma_pers(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    float* C, int ldc, __nv_bfloat16* Cb, int M, int N, int K, float alpha,
                    float beta, const float* __restrict__ bias, int act, int* err) {
  constexpr int A_BYTES = BM * TBK * 2;
  constexpr int B_BYTES = BN * TBK * 2;
  constexpr uint32_t TCOLS = 2 * BN;  // two accumulators of BN FP32 columns
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + TSTAGES * A_BYTES;
  __shared__ __align__(8) uint64_t full[TSTAGES], empty[TSTAGES], tfull[2], tempty[2];
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
  const int tiles = tiles_m * tiles_n;
  const int ktiles = (K + TBK - 1) / TBK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < TSTAGES; s++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])) : "memory");
    }
    for (int b = 0; b < 2; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&tfull[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(smem_u32(&tempty[b])) : "memory");
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  volatile int* abort = &abort_flag;
  bool ok = true;
  long long issued = 0;  // producer: ring steps whose loads were issued
  if (warp == 0) {
    if (lane == 0) {
      long long it = 0;
      for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        int mt, nt;
        tile_coords(t, tiles_m, tiles_n, mt, nt);
        for (int kt = 0; kt < ktiles; kt++, it++) {
          const int s = (int)(it % TSTAGES);
          if (it >= TSTAGES &&
              !mbar_wait_abort(smem_u32(&empty[s]), (uint32_t)((it / TSTAGES) - 1) & 1u, abort)) {
            ok = false;
            break;
          }
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                           smem_u32(&full[s])),
                       "r"(A_BYTES + B_BYTES)
                       : "memory");
          tma_load_2d(smem_u32(sA + s * A_BYTES), &tmA, kt * TBK, mt * BM, smem_u32(&full[s]));
          tma_load_2d(smem_u32(sB + s * B_BYTES), &tmB, kt * TBK, nt * BN, smem_u32(&full[s]));
          issued = it + 1;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = instr_desc(BM, BN);
      long long it = 0;
      int j = 0;
      for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, j++) {
        const int b = j & 1;
        if (j >= 2 && !mbar_wait_abort(smem_u32(&tempty[b]), (uint32_t)((j >> 1) - 1) & 1u, abort)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t acc_tmem = tmem + (uint32_t)(b * BN);
        for (int kt = 0; kt < ktiles; kt++, it++) {
          const int s = (int)(it % TSTAGES);
          if (!mbar_wait_abort(smem_u32(&full[s]), (uint32_t)(it / TSTAGES) & 1u, abort)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
          for (int kk = 0; kk < TBK / 16; kk++) {
            const uint64_t da = desc_sw128(smem_u32(sA + s * A_BYTES) + kk * 32);
            const uint64_t db = desc_sw128(smem_u32(sB + s * B_BYTES) + kk * 32);
            const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc_tmem),
                "l"(da), "l"(db), "r"(idesc), "r"(acc)
                : "memory");
          }
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                  smem_u32(&empty[s]))
              : "memory");
        }
        if (!ok) break;
        // the accumulator is complete once every MMA issued so far has finished
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&tfull[b]))
            : "memory");
      }
    }
  } else {
    const int q = warp & 3;  // TMEM lanes 32 q .. 32 q + 31 (a warp's accessible quarter)
    int j = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, j++) {
      const int b = j & 1;
      if (!mbar_wait_abort(smem_u32(&tfull[b]), (uint32_t)(j >> 1) & 1u, abort)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      int mt, nt;
      tile_coords(t, tiles_m, tiles_n, mt, nt);
      const int row = mt * BM + q * 32 + lane;
      const int n0 = nt * BN;
#pragma unroll 1
      for (int c = 0; c < BN; c += 16) {
        uint32_t r[16];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + c);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
            "%11, %12, %13, %14, %15}, [%16];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (row < M) {
          float v[16];
#pragma unroll
          for (int jj = 0; jj < 16; jj++) {
            const int col = n0 + c + jj;
            v[jj] = alpha * __uint_as_float(r[jj]);
            if (col < N) {
              if (beta != 0.f) v[jj] += beta * C[(size_t)row * ldc + col];
              if (bias) v[jj] += bias[col];
              if (act == 1) v[jj] = tanhf(v[jj]);
            }
          }
          float* crow = C + (size_t)row * ldc + n0 + c;
          if (n0 + c + 16 <= N && (reinterpret_cast<uintptr_t>(crow) & 15) == 0) {
#pragma unroll
            for (int k4 = 0; k4 < 4; k4++)
              reinterpret_cast<float4*>(crow)[k4] =
                  make_float4(v[4 * k4], v[4 * k4 + 1], v[4 * k4 + 2], v[4 * k4 + 3]);
          } else {
#pragma unroll
            for (int jj = 0; jj < 16; jj++)
              if (n0 + c + jj < N) crow[jj] = v[jj];
          }
          if (Cb)
#pragma unroll
            for (int jj = 0; jj < 16; jj++)
              if (n0 + c + jj < N) Cb[(size_t)row * ldc + n0 + c + jj] = __float2bfloat16(v[jj]);
        }
      }
      // this warp's quarter of the accumulator is read: hand it back to the MMA issuer
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(&tempty[b]))
                     : "memory");
    }
  }
  ok = __syncthreads_and(ok) != 0;
  if (!ok) {
    // let the TMA loads still in flight land before the shared memory goes away
    if (warp == 0 && lane == 0)
      for (long long it = issued > TSTAGES ? issued - TSTAGES : 0; it < issued; it++)
        mbar_wait(smem_u32(&full[it % TSTAGES]), (uint32_t)(it / TSTAGES) & 1u);
    if (tid == 0) atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCOLS)
                 : "memory");
}

// C = alpha sum_z partial[z] (z in order) + beta C + bias, then tanh; BF16 copy.
__global__ void k_splitk_reduce(const float* partial, int splits, float* C, int ldc,
                                __nv_bfloat16* Cb, int M, int N, float alpha, float beta,
                                const float* bias, int act) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)M * N) return;
  const int row = (int)(i / N), col = (int)(i % N);
  float acc = 0.f;
  for (int z = 0; z < splits; z++) acc += partial[(size_t)z * M * N + i];
  float v = alpha * acc;
  if (beta != 0.f) v += beta * C[(size_t)row * ldc + col];
  if (bias) v += bias[col];
  if (act == 1) v = tanhf(v);
  C[(size_t)row * ldc + col] = v;
  if (Cb) Cb[(size_t)row * ldc + col] = __float2bfloat16(v);
}

// split-K workspaces, grown on demand, one per (device, stream): calls on different
// streams never share one, so they may run concurrently (the stream orders the calls
// that do share one).  At most kMaxWorkspaces are kept per device; a new stream beyond
// that frees the device's others first.  A caller holds g_ws_mu from the lookup until
// its kernels are enqueued, and cudaFree synchronises the device, so no workspace is
// freed while a call still uses it.
struct Workspace {
  float* p = nullptr;
  size_t size = 0;
};
constexpr size_t kMaxWorkspaces = 32;
std::mutex g_ws_mu;
std::map<std::pair<int, cudaStream_t>, Workspace> g_ws;

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn tensor_map_encoder() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// 2-D map of a row-major BF16 matrix [rows x K] (leading dimension ld), boxes of
// box_rows x 64 with the 128-byte swizzle; out-of-range elements read as zero.
bool make_tile_map(CUtensorMap* map, const void* base, int rows, int K, int ld, int box_rows) {
  const EncodeTiledFn enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)TBK, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
             es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
constexpr int tma_smem_bytes() {
  return TSTAGES * (BM * TBK * 2 + BN * TBK * 2) + 1024;
}

template <int BN>
cudaError_t launch_tma(const CUtensorMap& ta, const CUtensorMap& tb, dim3 grid, cudaStream_t st,
                       float* C, int ldc, __nv_bfloat16* Cb, int M, int N, int K, float alpha,
                       float beta, const float* bias, int act, int* err, int k_chunk,
                       float* partial) {
  static bool configured[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    const cudaError_t e = cudaFuncSetAttribute(
        k_gemm_tma<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, tma_smem_bytes<BN>());
    if (e != cudaSuccess) return e;
    configured[dev] = true;
  }
  k_gemm_tma<BN><<<grid, 128, tma_smem_bytes<BN>(), st>>>(ta, tb, C, ldc, Cb, M, N, K, alpha, beta,
                                                         bias, act, err, k_chunk, partial);
  return cudaGetLastError();
}

int num_sms() {
  static int n[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (!n[dev]) cudaDeviceGetAttribute(&n[dev], cudaDevAttrMultiProcessorCount, dev);
  return n[dev] > 0 ? n[dev] : 1;
}

template <int BN>
cudaError_t launch_tma_pers(const CUtensorMap& ta, const CUtensorMap& tb, cudaStream_t st, float* C,
                            int ldc, __nv_bfloat16* Cb, int M, int N, int K, float alpha,
                            float beta, const float* bias, int act, int* err) {
  static bool configured[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    const cudaError_t e = cudaFuncSetAttribute(
        k_gemm_tma_pers<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, tma_smem_bytes<BN>());
    if (e != cudaSuccess) return e;
    configured[dev] = true;
  }
  const int tiles = ((M + BM - 1) / BM) * ((N + BN - 1) / BN);
  const int grid = std::min(tiles, num_sms());
  k_gemm_tma_pers<BN><<<grid, PERS_THREADS, tma_smem_bytes<BN>(), st>>>(
      ta, tb, C, ldc, Cb, M, N, K, alpha, beta, bias, act, err);
  return cudaGetLastError();
}

// Tiny products (the plastic-strain network's 64-wide layers) on the CUDA cores: one
// thread per output, the BF16 operands' products summed in FP32 in K order, then the
// epilogue of the tensor-core kernels (alpha, beta, bias, tanh, BF16 copy).
__global__ void __launch_bounds__(256) k_gemm_small(const __nv_bfloat16* A, int lda, int tA,
                                                    const __nv_bfloat16* B, int ldb, int tB,
                                                    float* C, int ldc, __nv_bfloat16* Cb, int M,
                                                    int N, int K, float alpha, float beta,
                                                    const float* bias, int act) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)M * N) return;
  const int row = (int)(i / N), col = (int)(i % N);
  float acc = 0.f;
  for (int k = 0; k < K; k++) {
    const float a = __bfloat162float(tA ? A[(size_t)k * lda + row] : A[(size_t)row * lda + k]);
    const float b = __bfloat162float(tB ? B[(size_t)col * ldb + k] : B[(size_t)k * ldb + col]);
    acc = fmaf(a, b, acc);
  }
  float v = alpha * acc;
  if (beta != 0.f) v += beta * C[(size_t)row * ldc + col];
  if (bias) v += bias[col];
  if (act == 1) v = tanhf(v);
  C[(size_t)row * ldc + col] = v;
  if (Cb) Cb[(size_t)row * ldc + col] = __float2bfloat16(v);
}

}  // namespace

extern "C" int ci_gemm_bf16(const void* A, int lda, int transA, const void* B, int ldb, int transB,
                            float* C, int ldc, void* C_bf16, int M, int N, int K, float alpha,
                            float beta, const float* bias, int activation, int* d_error,
                            void* stream) {
  if (!A || !B || !C || !d_error || M <= 0 || N <= 0 || K <= 0)
    return ci::set_last_error(CI_ERR_INVALID, "ci_gemm_bf16: null pointer or empty shape");
  if (activation != 0 && activation != 1)
    return ci::set_last_error(CI_ERR_INVALID, "ci_gemm_bf16: activation must be 0 or 1");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // A B^T with both operands K-major and TMA-compatible rows: the pipelined kernel
  const bool tma_shape = !transA && transB && M >= BM && N >= 16 && K >= TBK && lda >= K &&
                         ldb >= K && lda % 8 == 0 && ldb % 8 == 0 &&
                         reinterpret_cast<uintptr_t>(A) % 16 == 0 &&
                         reinterpret_cast<uintptr_t>(B) % 16 == 0;
  // other shapes of at most 2^20 multiply-adds (a 64-wide layer, a single output column):
  // CUDA cores, where a 128-row tile pipeline would cost more than the product
  if (!tma_shape && (long long)M * N * K <= (1LL << 20)) {
    const long long outs = (long long)M * N;
    k_gemm_small<<<(unsigned)((outs + 255) / 256), 256, 0, st>>>(
        static_cast<const __nv_bfloat16*>(A), lda, transA, static_cast<const __nv_bfloat16*>(B),
        ldb, transB, C, ldc, static_cast<__nv_bfloat16*>(C_bf16), M, N, K, alpha, beta, bias,
        activation);
    return cudaGetLastError() == cudaSuccess
               ? CI_OK
               : ci::set_last_error(CI_ERR_CUDA, "ci_gemm_bf16: small-product launch failed");
  }
  bool tma = tma_shape;
  const int bn_tma = N <= 64 ? 64 : N <= 128 ? 128 : 256;
  CUtensorMap ta, tb;
  tma = tma && make_tile_map(&ta, A, M, K, lda, BM) && make_tile_map(&tb, B, N, K, ldb, bn_tma);
  const int bn = tma ? bn_tma : (N <= 64 ? 64 : 128);
  const int tiles = ((M + BM - 1) / BM) * ((N + bn - 1) / bn);
  // split K when the output has too few tiles to fill the GPU and K is long
  int splits = 1;
  if (tiles < 304 && K >= 8 * BK) splits = std::min((304 + tiles - 1) / tiles, (K + 4 * BK - 1) / (4 * BK));
  splits = std::max(1, std::min(splits, 512));
  int k_chunk = (K + splits - 1) / splits;
  k_chunk = (k_chunk + BK - 1) / BK * BK;
  splits = (K + k_chunk - 1) / k_chunk;
  float* partial = nullptr;
  std::unique_lock<std::mutex> ws_lock(g_ws_mu, std::defer_lock);  // held until enqueued
  if (splits > 1) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
      return ci::set_last_error(CI_ERR_CUDA, "ci_gemm_bf16: no current device");
    const size_t need = sizeof(float) * (size_t)splits * M * N;
    ws_lock.lock();
    if (!g_ws.count({dev, st})) {
      size_t on_dev = 0;
      for (const auto& kv : g_ws) on_dev += kv.first.first == dev;
      if (on_dev >= kMaxWorkspaces)
        for (auto it = g_ws.begin(); it != g_ws.end();) {
          if (it->first.first == dev) {
            if (it->second.p) cudaFree(it->second.p);
            it = g_ws.erase(it);
          } else {
            ++it;
          }
        }
    }
    Workspace& w = g_ws[{dev, st}];
    if (w.size < need) {
      if (w.p) cudaFree(w.p);  // synchronises the device: no call still reads it
      w.p = nullptr;
      w.size = 0;
      if (cudaMalloc(&w.p, need) != cudaSuccess)
        return ci::set_last_error(CI_ERR_NOMEM, "ci_gemm_bf16: split-K workspace");
      w.size = need;
    }
    partial = w.p;
  }
  dim3 grid((M + BM - 1) / BM, (N + bn - 1) / bn, splits);
  __nv_bfloat16* cb = static_cast<__nv_bfloat16*>(C_bf16);
  cudaError_t le = cudaSuccess;
  if (tma && splits == 1) {
    if (bn == 64)
      le = launch_tma_pers<64>(ta, tb, st, C, ldc, cb, M, N, K, alpha, beta, bias, activation, d_error);
    else if (bn == 128)
      le = launch_tma_pers<128>(ta, tb, st, C, ldc, cb, M, N, K, alpha, beta, bias, activation, d_error);
    else
      le = launch_tma_pers<256>(ta, tb, st, C, ldc, cb, M, N, K, alpha, beta, bias, activation, d_error);
    if (le != cudaSuccess) return ci::set_last_error(CI_ERR_CUDA, cudaGetErrorString(le));
  } else if (tma) {
    if (bn == 64)
      le = launch_tma<64>(ta, tb, grid, st, C, ldc, cb, M, N, K, alpha, beta, bias, activation,
                          d_error, k_chunk, partial);
    else if (bn == 128)
      le = launch_tma<128>(ta, tb, grid, st, C, ldc, cb, M, N, K, alpha, beta, bias, activation,
                           d_error, k_chunk, partial);
    else
      le = launch_tma<256>(ta, tb, grid, st, C, ldc, cb, M, N, K, alpha, beta, bias, activation,
                           d_error, k_chunk, partial);
    if (le != cudaSuccess) return ci::set_last_error(CI_ERR_CUDA, cudaGetErrorString(le));
  } else if (bn == 64) {
    k_gemm_bf16<64><<<grid, 128, 0, st>>>(
        static_cast<const __nv_bfloat16*>(A), lda, transA, static_cast<const __nv_bfloat16*>(B),
        ldb, transB, C, ldc, cb, M, N, K, alpha, beta, bias, activation, d_error, k_chunk, partial);
  } else {
    k_gemm_bf16<128><<<grid, 128, 0, st>>>(
        static_cast<const __nv_bfloat16*>(A), lda, transA, static_cast<const __nv_bfloat16*>(B),
        ldb, transB, C, ldc, cb, M, N, K, alpha, beta, bias, activation, d_error, k_chunk, partial);
  }
  if (splits > 1) {
    const long long mn = (long long)M * N;
    k_splitk_reduce<<<(unsigned)((mn + 255) / 256), 256, 0, st>>>(partial, splits, C, ldc, cb, M, N,
                                                                  alpha, beta, bias, activation);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ci::set_last_error(CI_ERR_CUDA, cudaGetErrorString(e));
  return CI_OK;
}
