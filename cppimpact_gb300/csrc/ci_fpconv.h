// ci_fpconv.h -- FP64 <-> FP32 conversions on the integer pipe.
//
// On GB300 the FP64 unit of an SM retires 2 thread operations per clock, and a format
// conversion between FP64 and FP32 occupies it like a DFMA.  The nodal update converts
// three FP32 accelerations to FP64 and six FP64 state values to FP32 copies per node and
// step; done with a handful of 32-bit integer operations each, those conversions leave
// the FP64 unit to the six DFMAs of the update (measured: the staging phase of the fused
// step keeps the FP64 unit 68 % busy with hardware conversions).
//
// Both functions give the bits of the hardware conversion (round to nearest, ties to
// even) for every input: the FP32 normal range and signed zeros take the integer path;
// the rare rest (FP32 subnormals, overflow, infinities, NaNs) falls back to the
// hardware conversion.  They compile for host and device, so the host tests check the
// integer path bit for bit against the host's own conversions.
#ifndef CI_FPCONV_H
#define CI_FPCONV_H

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define CI_HD __host__ __device__ __forceinline__
#else
#define CI_HD inline
#endif

namespace ci {

CI_HD uint64_t fp_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

CI_HD uint32_t fp_bits(float x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

CI_HD double fp_f64(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, sizeof(x));
  return x;
#endif
}

CI_HD float fp_f32(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, sizeof(x));
  return x;
#endif
}

// (float)x, round to nearest even.
CI_HD float f64_to_f32(double x) {
  const uint64_t b = fp_bits(x);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t s = hi & 0x80000000u;
  const uint32_t e = (hi >> 20) & 0x7ffu;  // biased FP64 exponent
  if (e - 897u <= 253u) {                  // 897 <= e <= 1150: FP32 exponent 1..254
    // 23 kept mantissa bits and the 29 dropped ones
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1fffffffu;
    const uint32_t up = (rem > 0x10000000u) | ((rem == 0x10000000u) & (m & 1u));
    return fp_f32(s | (((e - 896u) << 23) + m + up));  // a mantissa carry bumps the exponent
  }
  if (((hi & 0x7fffffffu) | lo) == 0u) return fp_f32(s);  // +-0
  return (float)x;
}

// (double)x, exact.
CI_HD double f32_to_f64(float x) {
  const uint32_t a = fp_bits(x);
  const uint32_t s = a & 0x80000000u, m = a & 0x7fffffffu;
  if (m - 0x00800000u < 0x7f000000u) {  // normal: exponent rebias 127 -> 1023
    const uint32_t hi = s | ((m >> 3) + 0x38000000u);
    return fp_f64(((uint64_t)hi << 32) | (uint32_t)(m << 29));
  }
  if (m == 0u) return fp_f64((uint64_t)s << 32);  // +-0
  return (double)x;
}

}  // namespace ci

#endif
