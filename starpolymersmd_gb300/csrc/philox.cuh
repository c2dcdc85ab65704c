// Counter-based random numbers for the collision step, device side.
//
// Generator: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies
// (0xD2511F53, 0xCD9E8D57) with Weyl key schedule (0x9E3779B9, 0xBB67AE85).
// Stream layout (one block = one Philox call = four 32-bit words w0..w3):
//   key              = { lo32(seed), hi32(seed) }         per replica
//   counter(c, s, k) = { c, lo32(s), hi32(s), k }          c = cell in replica,
//                                                          s = collision counter
//   double uniforms  uA = U53(w0, w1), uB = U53(w2, w3),
//                    U53(lo, hi) = ((hi:lo) >> 11) * 2^-53 + 2^-54  in (0, 1)
//   float uniforms   uA = (w1 >> 9) * 2^-23 + 2^-24, uB from w3: the same top bits
//   block k = 0            -> (u_phi, u_theta) of the rotation axis
//   blocks 1+2i, 2+2i      -> iteration i of the gamma sampler (normal, acceptance)
//   cell c = 0xFFFFFFFF    -> grid shift: block 0 gives x, y; block 1 gives z
// Gamma(a >= 1): Marsaglia & Tsang, "A simple method for generating gamma
// variables", ACM TOMS 26(3), 2000, with a Box-Muller normal
// z = sqrt(-2 ln uA) cos(2 pi uB).
#pragma once
#include <stdint.h>

#include "precision.cuh"

namespace smpc {

struct Philox4 {
  uint32_t w[4];
};

__device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                 uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t lo1 = 0xCD9E8D57u * c2;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  Philox4 out;
  out.w[0] = c0;
  out.w[1] = c1;
  out.w[2] = c2;
  out.w[3] = c3;
  return out;
}

template <typename R>
struct Uniform2 {
  R a, b;
};

__device__ __forceinline__ double u53(uint32_t lo, uint32_t hi) {
  const uint64_t bits = ((static_cast<uint64_t>(hi) << 32) | lo) >> 11;
  return __dadd_rn(__dmul_rn(static_cast<double>(bits), 0x1.0p-53), 0x1.0p-54);
}

// top 23 bits of the high word, built without a conversion instruction
__device__ __forceinline__ float u24(uint32_t hi) { return u23_open(hi); }

template <typename R>
__device__ __forceinline__ Uniform2<R> philox_uniforms(unsigned long long seed, uint32_t cell,
                                                       unsigned long long step, uint32_t k);

template <>
__device__ __forceinline__ Uniform2<double> philox_uniforms<double>(unsigned long long seed,
                                                                    uint32_t cell,
                                                                    unsigned long long step,
                                                                    uint32_t k) {
  const Philox4 b = philox4x32_10(cell, static_cast<uint32_t>(step),
                                  static_cast<uint32_t>(step >> 32), k,
                                  static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
  return Uniform2<double>{u53(b.w[0], b.w[1]), u53(b.w[2], b.w[3])};
}

template <>
__device__ __forceinline__ Uniform2<float> philox_uniforms<float>(unsigned long long seed,
                                                                  uint32_t cell,
                                                                  unsigned long long step,
                                                                  uint32_t k) {
  const Philox4 b = philox4x32_10(cell, static_cast<uint32_t>(step),
                                  static_cast<uint32_t>(step >> 32), k,
                                  static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
  return Uniform2<float>{u24(b.w[1]), u24(b.w[3])};
}

// Gamma(shape, 1) for shape >= 1 on the stream of (seed, cell, step).
// Returns false in *ok when the iteration limit was reached (the result is
// then the distribution's mode region value d, never used silently: callers
// raise ERR_GAMMA_ITERS).
template <typename R>
__device__ __forceinline__ R philox_gamma(unsigned long long seed, uint32_t cell,
                                          unsigned long long step, R shape, bool* ok) {
  const R third = R(1) / R(3);
  const R d = shape - third;
  const R c = R(1) / r_sqrt(R(9) * d);
  const R two_pi = R(6.283185307179586476925286766559);
  for (uint32_t it = 0; it < 64u; ++it) {
    const Uniform2<R> n = philox_uniforms<R>(seed, cell, step, 1u + 2u * it);
    const R x = r_sqrt(R(-2) * r_log(n.a)) * r_cos(two_pi * n.b);
    R v = R(1) + c * x;
    if (v <= R(0)) continue;
    v = v * v * v;
    const R u = philox_uniforms<R>(seed, cell, step, 2u + 2u * it).a;
    const R x2 = x * x;
    if (u < R(1) - R(0.0331) * (x2 * x2)) {
      *ok = true;
      return d * v;
    }
    if (r_log(u) < R(0.5) * x2 + d * (R(1) - v + r_log(v))) {
      *ok = true;
      return d * v;
    }
  }
  *ok = false;
  return d;
}

}  // namespace smpc
