// Precision-typed math for templated device code. Each helper is overloaded
// for float and double and calls the function of that precision explicitly,
// so FP32 code never promotes to double (a promoted call such as round(float)
// would run on the FP64 pipe, which is narrow on GB300).
#pragma once
#include <stdint.h>

namespace smpc {

__device__ __forceinline__ float r_round(float x) { return roundf(x); }
__device__ __forceinline__ double r_round(double x) { return ::round(x); }
__device__ __forceinline__ float r_floor(float x) { return floorf(x); }
__device__ __forceinline__ double r_floor(double x) { return ::floor(x); }
__device__ __forceinline__ float r_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double r_sqrt(double x) { return ::sqrt(x); }
__device__ __forceinline__ float r_log(float x) { return logf(x); }
__device__ __forceinline__ double r_log(double x) { return ::log(x); }
__device__ __forceinline__ float r_cos(float x) { return cosf(x); }
__device__ __forceinline__ double r_cos(double x) { return ::cos(x); }
__device__ __forceinline__ void r_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void r_sincos(double x, double* s, double* c) { ::sincos(x, s, c); }
__device__ __forceinline__ float r_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double r_fabs(double x) { return ::fabs(x); }
__device__ __forceinline__ bool r_isfinite(float x) { return isfinite(x); }
__device__ __forceinline__ bool r_isfinite(double x) { return isfinite(x); }

}  // namespace smpc

namespace smpc {

// ---------------------------------------------------------------------------
// float <-> int without conversion instructions. On GB300 the F2I / I2F
// conversions issue on the FP64 pipe (a few lanes per clock per SM), so the
// FP32 hot loops build integers from float bit patterns instead, with plain
// FP32 adds in a directed or nearest rounding mode:
//   x + 1.5*2^23 rounded to nearest puts rn(x) in the low mantissa bits for
//   |x| < 2^22; x + 2^23 rounded down puts floor(x) there for 0 <= x < 2^23.
// All three are exact.

// rn(x) (ties to even) for |x| < 2^22.
__device__ __forceinline__ int f2i_rn_small(float x) {
  return __float_as_int(__fadd_rn(x, 12582912.0f)) - 0x4B400000;
}
// floor(x) for 0 <= x < 2^23.
__device__ __forceinline__ int f2i_floor_nonneg(float x) {
  return __float_as_int(__fadd_rd(x, 8388608.0f)) - 0x4B000000;
}
// (float)i for |i| < 2^22.
__device__ __forceinline__ float i2f_small(int i) {
  return __fsub_rn(__int_as_float(i + 0x4B400000), 12582912.0f);
}

// Range of the fixed-point conversions below: |v| < FIX32_LIMIT. They do not
// clamp. Callers keep the largest |v| they convert (one max per term, cheaper
// than a clamp) and raise ERR_FIXPOINT when it reaches the limit, since the
// sums are meaningless then; NaN terms leave the maximum alone and are caught
// by the non-finite check on the collided velocities.
constexpr float FIX32_LIMIT = 4095.0f;

// v * 2^32 rounded to an int64, |v| < 2^12: hi = rn(v * 2^10) and the exact
// remainder v * 2^10 - hi (|.| <= 1/2) scaled by 2^22 give the two parts.
__device__ __forceinline__ long long f2fix32(float v) {
  const float a = v * 1024.0f;
  const int hi = f2i_rn_small(a);
  const float r = __fsub_rn(a, i2f_small(hi));
  const int lo = f2i_rn_small(r * 4194304.0f);
  return static_cast<long long>(hi) * 4194304ll + lo;
}

// The same value as f2fix32, added to split accumulators: hi (units of 2^-10)
// and lo (units of 2^-32); the sum is hi * 2^22 + lo. Each part is added as
// the raw bit pattern of its magic-number float, 0x4B400000 + part, with
// wrap-around unsigned adds; fix32_join takes the n magic offsets back out.
// |hi| < 2^22 and |lo| <= 2^21 per term, so 512 terms cannot overflow the
// signed sums. Three FMAs and an add per term: v 2^10 is exact (a power of
// two), so fma(v, 2^10, magic) is rn(v 2^10) + magic, and
// fma(v, 2^10, -rn(v 2^10)) is the remainder exactly.
constexpr uint32_t FIX32_MAGIC_BITS = 0x4B400000u;
__device__ __forceinline__ void fix32_add(float v, uint32_t& hi_acc, uint32_t& lo_acc) {
  const float m = fmaf(v, 1024.0f, 12582912.0f);             // rn(v 2^10) in the low bits
  const float r = fmaf(v, 1024.0f, -__fsub_rn(m, 12582912.0f));  // v 2^10 - rn(v 2^10), exact
  const float l = fmaf(r, 4194304.0f, 12582912.0f);          // rn(r 2^22) in the low bits
  hi_acc += __float_as_uint(m);
  lo_acc += __float_as_uint(l);
}
__device__ __forceinline__ long long fix32_join(uint32_t hi_acc, uint32_t lo_acc, int n_terms) {
  const uint32_t off = static_cast<uint32_t>(n_terms) * FIX32_MAGIC_BITS;
  return static_cast<long long>(static_cast<int>(hi_acc - off)) * 4194304ll +
         static_cast<int>(lo_acc - off);
}

// int64 2^32 fixed point to float (three exact 21-bit pieces, one rounding).
__device__ __forceinline__ float fix32_to_f(long long a) {
  const int a0 = static_cast<int>(a & 0x1FFFFFll);
  const int a1 = static_cast<int>((a >> 21) & 0x1FFFFFll);
  const int a2 = static_cast<int>(a >> 42);
  const float hi = fmaf(i2f_small(a2), 2097152.0f, i2f_small(a1));
  return fmaf(hi, 2097152.0f, i2f_small(a0)) * 2.3283064365386963e-10f;
}

// Uniform in (0, 1) from the top 23 bits of w: the mantissa of a float in
// [1, 2) minus one, plus half a step.
__device__ __forceinline__ float u23_open(uint32_t w) {
  return __fadd_rn(__fsub_rn(__uint_as_float(0x3F800000u | (w >> 9)), 1.0f), 0x1.0p-24f);
}

}  // namespace smpc
