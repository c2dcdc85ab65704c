// FP32 fast-path collision kernels (the FP64 reference-parity path keeps the
// operation-by-operation kernels of mpc_kernels.cuh).
//
// Same physics as MPC::step (star-polymers/lib/Hydrodynamics/MPC.cpp:116-142),
// arranged for throughput on GB300:
//  * all per-replica constants come from a float frame written once per
//    collision (no double->float conversion in any thread: those issue on the
//    FP64 pipe, 2 lanes/clock/SM on this part);
//  * the reference's three Lees-Edwards wraps (after streaming, after the
//    grid shift, after the unshift, MPC.cpp:192-197, 301-311) are composed
//    exactly: with X = x + v h (unwrapped) the collision frame is the image
//    c_s = img(X_y + s_y) of the shifted point, the final position is the
//    image c_t = img(X_y) of the unshifted one, and the velocity picks up the
//    same total jump -(c_t) shear Ly, -(c_s) of it before the collision;
//  * k_collide takes every particle's cell from the counting sort itself
//    (sorted position -> cell range), so it never recomputes cell indices;
//  * float<->int work uses exact FP32-pipe constructions (precision.cuh).
#pragma once
#include <stdint.h>

#include "mpc_kernels.cuh"

namespace smpc {

// image index of y (-1, 0, +1) for |y| < 1.5 L; general rounding beyond
__device__ __forceinline__ float img_f(float y, float L, float half) {
  if (fabsf(y) < 1.5f * L) return y >= half ? 1.0f : (y < -half ? -1.0f : 0.0f);
  return rintf(__fdiv_rn(y, L));
}

// periodic wrap into [-L/2, L/2) for |x| < 2.5 L; general rounding beyond
__device__ __forceinline__ float wrap_f(float x, float L, float half) {
  if (!(fabsf(x) < 2.5f * L)) x = __fsub_rn(x, __fmul_rn(L, rintf(__fdiv_rn(x, L))));
  x = x >= half ? __fsub_rn(x, L) : (x < -half ? __fadd_rn(x, L) : x);
  return x >= half ? __fsub_rn(x, L) : (x < -half ? __fadd_rn(x, L) : x);
}

// The same two functions without their general-rounding branches, as
// selects: img_sel is img_f for |y| < 1.5 L, wrap_sel is wrap_f for
// |x| < 2.5 L, bit for bit (x - c L with c in {-1, 0, 1} is exact or one
// correctly rounded add either way).
__device__ __forceinline__ float img_sel(float y, float half) {
  return y >= half ? 1.0f : (y < -half ? -1.0f : 0.0f);
}
__device__ __forceinline__ float wrap_sel(float x, float L, float half) {
  x = fmaf(-img_sel(x, half), L, x);
  return fmaf(-img_sel(x, half), L, x);
}

// Recentre (MPC::check_bounds, MPC.cpp:183-188, incl. its LE wrap) and
// stream (MPC.cpp:194): X = x + v h, unwrapped. Explicitly rounded so the
// bin and collide kernels produce identical X.
__device__ __forceinline__ void stream_f(const FrameF& f, float4& x, float4& v) {
  if (f.recentre) {
    x.x = __fsub_rn(x.x, f.com[0]);
    x.y = __fsub_rn(x.y, f.com[1]);
    x.z = __fsub_rn(x.z, f.com[2]);
    v.x = __fsub_rn(v.x, f.comv[0]);
    v.y = __fsub_rn(v.y, f.comv[1]);
    v.z = __fsub_rn(v.z, f.comv[2]);
    if (f.shear_on) {
      const float c0 = img_f(x.y, f.L[1], f.half[1]);
      x.y = __fsub_rn(x.y, __fmul_rn(c0, f.L[1]));
      x.x = __fsub_rn(x.x, __fmul_rn(c0, f.delrx));
      v.x = __fsub_rn(v.x, __fmul_rn(c0, f.shearLy));
    }
  }
  x.x = __fadd_rn(x.x, __fmul_rn(v.x, f.h));
  x.y = __fadd_rn(x.y, __fmul_rn(v.y, f.h));
  x.z = __fadd_rn(x.z, __fmul_rn(v.z, f.h));
}

// Shifted collision-frame position and its y image index.
__device__ __forceinline__ float shifted_f(const FrameF& f, const float4& X, float& xs, float& ys,
                                           float& zs) {
  ys = __fadd_rn(X.y, f.shift[1]);
  const float cs = f.shear_on ? img_f(ys, f.L[1], f.half[1]) : 0.0f;
  if (f.shear_on) {
    ys = __fsub_rn(ys, __fmul_rn(cs, f.L[1]));
    xs = wrap_f(__fsub_rn(__fadd_rn(X.x, f.shift[0]), __fmul_rn(cs, f.delrx)), f.L[0], f.half[0]);
  } else {
    ys = wrap_f(ys, f.L[1], f.half[1]);
    xs = wrap_f(__fadd_rn(X.x, f.shift[0]), f.L[0], f.half[0]);
  }
  zs = wrap_f(__fadd_rn(X.z, f.shift[2]), f.L[2], f.half[2]);
  return cs;
}

__device__ __forceinline__ uint32_t cell_f(const FrameF& f, float x, float y, float z) {
  const int ix = min(f2i_floor_nonneg(fmaxf(__fadd_rn(x, f.half[0]), 0.0f)), f.Li[0] - 1);
  const int iy = min(f2i_floor_nonneg(fmaxf(__fadd_rn(y, f.half[1]), 0.0f)), f.Li[1] - 1);
  const int iz = min(f2i_floor_nonneg(fmaxf(__fadd_rn(z, f.half[2]), 0.0f)), f.Li[2] - 1);
  return static_cast<uint32_t>(ix + f.Li[0] * (iy + f.Li[1] * iz));
}

__device__ __forceinline__ float4 ld_f4(const float* p, size_t i) {
  return __ldg(reinterpret_cast<const float4*>(p) + i);
}
__device__ __forceinline__ void st_f4(float* p, size_t i, float4 v) {
  reinterpret_cast<float4*>(p)[i] = v;
}

// --------------------------------------------------------------- binning

// PACKED: 32-bit keys (local cell << 16 | rank) for contexts whose boxes
// have at most 65,536 cells each, half the bytes of the (global cell, rank)
// pairs between the binning and the permutation. A cell of 65,535 particles
// or more cannot be packed and raises ERR_KEY_MISMATCH.
template <int NT, int U, bool PACKED>
__global__ void __launch_bounds__(NT) k_fluid_bin_f32(const Tile* tiles, const RepInfo* reps,
                                                      const FrameF* frames,
                                                      const float* __restrict__ st,
                                                      uint2* __restrict__ keys, uint32_t* count,
                                                      ErrorState* err) {
  const Tile t = tiles[blockIdx.x];
  const FrameF f = frames[t.rep];
  const uint32_t cbase = static_cast<uint32_t>(reps[t.rep].cell_base);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  for (int base = t.begin; base < t.end; base += NT * U) {
    float4 x[U], v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = base + u * NT + threadIdx.x;
      if (i < t.end) {
        x[u] = ld_f4(st, 2 * static_cast<size_t>(i));
        v[u] = ld_f4(st, 2 * static_cast<size_t>(i) + 1);
      }
    }
    uint32_t key[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = base + u * NT + threadIdx.x;
      key[u] = KEY_NONE;
      if (i < t.end && __float_as_uint(x[u].w) != SLOT_EMPTY) {
        stream_f(f, x[u], v[u]);
        float xs, ys, zs;
        shifted_f(f, x[u], xs, ys, zs);
        key[u] = cbase + cell_f(f, xs, ys, zs);
      }
    }
    unsigned peers[U];
    uint32_t rbase[U];
#pragma unroll
    for (int u = 0; u < U; ++u) peers[u] = __match_any_sync(0xFFFFFFFFu, key[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      rbase[u] = 0u;
      if (lane == static_cast<unsigned>(__ffs(peers[u]) - 1) && key[u] != KEY_NONE)
        rbase[u] = atomicAdd(count + key[u], __popc(peers[u]));
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t b0 = __shfl_sync(0xFFFFFFFFu, rbase[u], __ffs(peers[u]) - 1);
      const int i = base + u * NT + threadIdx.x;
      if (i >= t.end) continue;
      const uint32_t rank = b0 + __popc(peers[u] & below);
      if (PACKED) {
        uint32_t k32 = KEY_NONE;
        if (key[u] != KEY_NONE) {
          if (rank >= 0xFFFFu)
            raise_error(err, ERR_KEY_MISMATCH, static_cast<uint32_t>(i), key[u]);
          else
            k32 = ((key[u] - cbase) << 16) | rank;
        }
        reinterpret_cast<uint32_t*>(keys)[i] = k32;
      } else {
        keys[i] = make_uint2(key[u], rank);
      }
    }
  }
}

// --------------------------------------------------------------- collide

constexpr size_t collide_f32_dyn_smem(int cap) {
  return static_cast<size_t>(cap) * (2 * sizeof(float4) + sizeof(short));
}

// A staged particle: sx = (X unwrapped streamed position, id or MONO_BIT|m),
// sv = (velocity in the collision frame, mass).
struct FastP {
  float4 x;
  float4 v;
};

__device__ __forceinline__ void fetch_f(FastP& P, uint32_t src, const float* st,
                                        const float* mpos, const float* mvel, const int* mimg,
                                        const FrameF& f, int wrap_mono) {
  if (src & MONO_BIT) {
    const uint32_t m = src & ~MONO_BIT;
    P.v = reinterpret_cast<const float4*>(mvel)[m];
    P.v.w = reinterpret_cast<const float4*>(mpos)[m].w;
    if (wrap_mono == MONOBIN_WRAPPED)
      P.v.x = __fsub_rn(P.v.x, __fmul_rn(i2f_small(mimg[m]), f.shearLy));
    P.x = make_float4(0.f, 0.f, 0.f, __uint_as_float(src));
  } else {
    P.x = ld_f4(st, 2 * static_cast<size_t>(src));
    P.v = ld_f4(st, 2 * static_cast<size_t>(src) + 1);
  }
}

// Solvent: stream (the unwrapped X replaces the position, the id stays in
// .w) and move the velocity into the shifted collision frame (image c_s).
// Monomers keep what fetch_f loaded.
__device__ __forceinline__ void frame_f(FastP& P, const FrameF& f, float solvent_mass) {
  if (__float_as_uint(P.x.w) & MONO_BIT) return;
  stream_f(f, P.x, P.v);
  if (f.shear_on) {
    const float cs = img_f(__fadd_rn(P.x.y, f.shift[1]), f.L[1], f.half[1]);
    P.v.x = __fsub_rn(P.v.x, __fmul_rn(cs, f.shearLy));
  }
  P.v.w = solvent_mass;
}

// Per-tile work shared by the collide kernels. Staged particles sit in
// s_x/s_v[0, nloc) in sorted order; sorted position p0 + j belongs to the
// tile's local cell lc with s_off[lc] <= p0 + j < s_off[lc + 1]. Entries at
// nloc and beyond (a tile fuller than the staging capacity) are read from
// global memory again.
struct CollideF32Args {
  const float* st_in;
  float* st_out;
  const float* mpos;
  float* mvel;
  const int* mimg;
  const uint32_t* perm;
  const double* inj_gamma;
  const double* inj_uphi;
  const double* inj_utheta;
  int rng;
  int mono_bin;
  ErrorState* err;
};

// cells: two lanes per cell; int64 2^32 fixed-point sums (exact, order-free),
// then the thermostat scale and the rotation (folded together) per cell
template <int NT>
__device__ __forceinline__ void collide_cells_f32(const CollideF32Args& A, const FrameF& f,
                                                  const Tile& t, const uint32_t* s_off, int nc,
                                                  uint32_t p0, int nloc, const float4* s_x,
                                                  const float4* s_v, short* s_lc, float4* s_rc,
                                                  unsigned long long seed,
                                                  unsigned long long step, uint32_t cbase) {
  const float* st_in = A.st_in;
  const float* mpos = A.mpos;
  const float* mvel = A.mvel;
  const int* mimg = A.mimg;
  const uint32_t* perm = A.perm;
  const int mono_bin = A.mono_bin;
  const int rng = A.rng;
  const double* inj_gamma = A.inj_gamma;
  const double* inj_uphi = A.inj_uphi;
  const double* inj_utheta = A.inj_utheta;
  ErrorState* err = A.err;
  {
    const int lc = threadIdx.x >> 1;
    const int half = threadIdx.x & 1;
    const bool live = lc < nc;
    const int j0 = live ? static_cast<int>(s_off[lc] - p0) : 0;
    const int j1 = live ? static_cast<int>(s_off[lc + 1] - p0) : 0;
    // One pass: P = sum m v and S = sum m |v|^2, both int64 fixed point (exact
    // and independent of the particles' order), then c = P / M and
    // E = (S - |P|^2 / M) / 2. S is kept at 2^24 fixed point (the m |v|^2
    // terms are pre-scaled by 2^-8) so fast shear flows stay in range; the
    // one float subtraction costs ~1e-5 relative in E at a cell velocity of
    // ten thermal speeds.
    long long px = 0, py = 0, pz = 0, e = 0;
    int nsol = 0;
    float mmono = 0.0f;
    float big = 0.0f;  // largest fixed-point term (range check)
    if (j1 - j0 <= 1024) {
      // at most 512 terms per lane: 32-bit split accumulators
      uint32_t xh = 0, xl = 0, yh = 0, yl = 0, zh = 0, zl = 0, eh = 0, el = 0;
      int terms = 0;
      for (int j = j0 + half; j < j1; j += 2) {
        float4 v, x;
        if (j < nloc) {
          v = s_v[j];
          x = s_x[j];
          s_lc[j] = static_cast<short>(lc);
        } else {  // past the staging capacity: straight from global memory
          FastP P;
          fetch_f(P, perm[p0 + j], st_in, mpos, mvel, mimg, f, mono_bin);
          frame_f(P, f, f.solvent_mass);
          v = P.v;
          x = P.x;
        }
        const float mx = v.x * v.w, my = v.y * v.w, mz = v.z * v.w;
        const float et = (v.w * 0.00390625f) * (v.x * v.x + v.y * v.y + v.z * v.z);
        big = fmaxf(big, fmaxf(fmaxf(fabsf(mx), fabsf(my)), fmaxf(fabsf(mz), et)));
        fix32_add(mx, xh, xl);
        fix32_add(my, yh, yl);
        fix32_add(mz, zh, zl);
        fix32_add(et, eh, el);
        ++terms;
        if (__float_as_uint(x.w) & MONO_BIT) {
          mmono += v.w;
        } else {
          ++nsol;
        }
      }
      px = fix32_join(xh, xl, terms);
      py = fix32_join(yh, yl, terms);
      pz = fix32_join(zh, zl, terms);
      e = fix32_join(eh, el, terms);
    } else {
      for (int j = j0 + half; j < j1; j += 2) {
        float4 v, x;
        if (j < nloc) {
          v = s_v[j];
          x = s_x[j];
          s_lc[j] = static_cast<short>(lc);
        } else {
          FastP P;
          fetch_f(P, perm[p0 + j], st_in, mpos, mvel, mimg, f, mono_bin);
          frame_f(P, f, f.solvent_mass);
          v = P.v;
          x = P.x;
        }
        const float mx = v.x * v.w, my = v.y * v.w, mz = v.z * v.w;
        const float et = (v.w * 0.00390625f) * (v.x * v.x + v.y * v.y + v.z * v.z);
        big = fmaxf(big, fmaxf(fmaxf(fabsf(mx), fabsf(my)), fmaxf(fabsf(mz), et)));
        px += f2fix32(mx);
        py += f2fix32(my);
        pz += f2fix32(mz);
        e += f2fix32(et);
        if (__float_as_uint(x.w) & MONO_BIT) {
          mmono += v.w;
        } else {
          ++nsol;
        }
      }
    }
    px += __shfl_xor_sync(0xFFFFFFFFu, px, 1);
    py += __shfl_xor_sync(0xFFFFFFFFu, py, 1);
    pz += __shfl_xor_sync(0xFFFFFFFFu, pz, 1);
    e += __shfl_xor_sync(0xFFFFFFFFu, e, 1);
    nsol += __shfl_xor_sync(0xFFFFFFFFu, nsol, 1);
    mmono += __shfl_xor_sync(0xFFFFFFFFu, mmono, 1);
    const float mt = fmaf(i2f_small(nsol), f.solvent_mass, mmono);
    const float inv = mt > 0.f ? 1.0f / mt : 0.0f;
    const float q0 = fix32_to_f(px), q1 = fix32_to_f(py), q2 = fix32_to_f(pz);
    const float cm0 = q0 * inv, cm1 = q1 * inv, cm2 = q2 * inv;
    const float ekin =
        fmaxf(0.5f * (fix32_to_f(e) * 256.0f - (q0 * q0 + q1 * q1 + q2 * q2) * inv), 0.0f);
    const uint32_t cg = static_cast<uint32_t>(t.begin + lc);
    const uint32_t cl = cg - cbase;
    const uint32_t nn = static_cast<uint32_t>(j1 - j0);
    if (big >= FIX32_LIMIT) raise_error(err, ERR_FIXPOINT, cg, __float_as_uint(big));
    float scale = -1.0f;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;  // rotation axis (lane 1)
    if (rng == RNG_INJECT) {
      if (half == 0) {
        if (live && nn >= 2u) {
          const float gv = static_cast<float>(inj_gamma[cg]);
          scale = ekin > 0.f ? sqrtf(gv / ekin) : 1.0f;
        }
      } else if (live) {
        const float uphi = static_cast<float>(inj_uphi[cg]);
        const float theta = 2.0f * (static_cast<float>(inj_utheta[cg]) - 0.5f);
        const float stt = sqrtf(1.0f - theta * theta);
        float sphi, cphi;
        sincosf(6.283185307179586f * uphi, &sphi, &cphi);
        a0 = stt * cphi;
        a1 = stt * sphi;
        a2 = theta;
      }
    } else {
      // Both lanes of a cell draw at once: lane 1 the axis block (k = 0),
      // lane 0 the first normal pair of the gamma sampler (k = 1); then one
      // r = sqrt(t), sincos(2 pi w) serves both (lane 0: t = -2 ln u_a,
      // w = u_b, normal r cos; lane 1: t = 1 - theta^2, w = u_phi, axis
      // (r cos, r sin, theta)). Same stream and formulas as philox_gamma /
      // philox_uniforms.
      const Philox4 b = philox4x32_10(cl, static_cast<uint32_t>(step),
                                      static_cast<uint32_t>(step >> 32), half ? 0u : 1u,
                                      static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
      const float ua = u24(b.w[1]), ub = u24(b.w[3]);
      const float theta = 2.0f * (ub - 0.5f);
      const float lg = logf(half ? 1.0f : ua);
      const float r = sqrtf(half ? 1.0f - theta * theta : -2.0f * lg);
      float sn, cs;
      sincosf(6.283185307179586f * (half ? ua : ub), &sn, &cs);
      if (half == 0) {
        if (live && nn >= 2u) {
          // Marsaglia-Tsang, iteration 0 with the normal above, further
          // iterations (rare) exactly as philox_gamma
          const float shape = 1.5f * i2f_small(static_cast<int>(nn - 1u));
          const float d = shape - 1.0f / 3.0f;
          const float c9 = 1.0f / sqrtf(9.0f * d);
          float x = r * cs;
          float gv = -1.0f;
          for (uint32_t it = 0; it < 64u; ++it) {
            if (it > 0) {
              const Uniform2<float> n2 = philox_uniforms<float>(seed, cl, step, 1u + 2u * it);
              x = sqrtf(-2.0f * logf(n2.a)) * cosf(6.283185307179586f * n2.b);
            }
            float v = 1.0f + c9 * x;
            if (v <= 0.0f) continue;
            v = v * v * v;
            const float u = philox_uniforms<float>(seed, cl, step, 2u + 2u * it).a;
            const float x2 = x * x;
            if (u < 1.0f - 0.0331f * (x2 * x2) || logf(u) < 0.5f * x2 + d * (1.0f - v + logf(v))) {
              gv = d * v;
              break;
            }
          }
          if (gv < 0.0f) {
            raise_error(err, ERR_GAMMA_ITERS, cg, nn);
            gv = d;
          }
          gv *= f.kT;
          scale = ekin > 0.f ? sqrtf(gv / ekin) : 1.0f;
        }
      } else {
        a0 = r * cs;
        a1 = r * sn;
        a2 = theta;
      }
    }
    float M[9];
    if (half == 1) {
      const float c = f.rot_c, s = f.rot_s;
      M[0] = a0 * a0 + (1.0f - a0 * a0) * c;
      M[1] = a0 * a1 * (1.0f - c) - a2 * s;
      M[2] = a0 * a2 * (1.0f - c) + a1 * s;
      M[3] = a0 * a1 * (1.0f - c) + a2 * s;
      M[4] = a1 * a1 + (1.0f - a1 * a1) * c;
      M[5] = a1 * a2 * (1.0f - c) - a0 * s;
      M[6] = a0 * a2 * (1.0f - c) - a1 * s;
      M[7] = a1 * a2 * (1.0f - c) + a0 * s;
      M[8] = a2 * a2 + (1.0f - a2 * a2) * c;
    }
    scale = __shfl_xor_sync(0xFFFFFFFFu, scale, 1);
    if (half == 1 && live) {
      const float sc = scale >= 0.0f ? scale : 1.0f;  // thermostat folded into R
      // row q of sR with component q of the cell's velocity in .w
      s_rc[3 * lc] = make_float4(M[0] * sc, M[1] * sc, M[2] * sc, cm0);
      s_rc[3 * lc + 1] = make_float4(M[3] * sc, M[4] * sc, M[5] * sc, cm1);
      s_rc[3 * lc + 2] = make_float4(M[6] * sc, M[7] * sc, M[8] * sc, cm2);
    }
  }
}

// apply: v' = cmv + sR (v - cmv), back to the primary box, write in cell order
template <int NT>
__device__ __forceinline__ void collide_apply_f32(const CollideF32Args& A, const FrameF& f,
                                                  const uint32_t* s_off, uint32_t p0, int n,
                                                  int nloc, const float4* s_x, const float4* s_v,
                                                  const short* s_lc, const float4* s_rc) {
  const float* st_in = A.st_in;
  float* st_out = A.st_out;
  const float* mpos = A.mpos;
  float* mvel = A.mvel;
  const int* mimg = A.mimg;
  const uint32_t* perm = A.perm;
  const int mono_bin = A.mono_bin;
  ErrorState* err = A.err;
  for (int j = threadIdx.x; j < n; j += NT) {
    float4 x, v;
    int lc;
    if (j < nloc) {
      x = s_x[j];
      v = s_v[j];
      lc = s_lc[j];
    } else {
      FastP P;
      fetch_f(P, perm[p0 + j], st_in, mpos, mvel, mimg, f, mono_bin);
      frame_f(P, f, f.solvent_mass);
      x = P.x;
      v = P.v;
      // cell of sorted position p0 + j: the range that contains it
      lc = 0;
      while (static_cast<int>(s_off[lc + 1] - p0) <= j) ++lc;
    }
    const float4 r0 = s_rc[3 * lc], r1 = s_rc[3 * lc + 1], r2 = s_rc[3 * lc + 2];
    const float d0 = v.x - r0.w, d1 = v.y - r1.w, d2 = v.z - r2.w;
    float vx = r0.w + (r0.x * d0 + r0.y * d1 + r0.z * d2);
    const float vy = r1.w + (r1.x * d0 + r1.y * d1 + r1.z * d2);
    const float vz = r2.w + (r2.x * d0 + r2.y * d1 + r2.z * d2);
    const uint32_t tag = __float_as_uint(x.w);
    if (!(isfinite(vx) && isfinite(vy) && isfinite(vz))) raise_error(err, ERR_NONFINITE, p0 + j, tag);
    const size_t p = static_cast<size_t>(p0) + j;
    if (tag & MONO_BIT) {
      const uint32_t m = tag & ~MONO_BIT;
      if (mono_bin == MONOBIN_WRAPPED) vx = __fadd_rn(vx, __fmul_rn(i2f_small(mimg[m]), f.shearLy));
      float4 mv = reinterpret_cast<float4*>(mvel)[m];
      mv.x = vx;
      mv.y = vy;
      mv.z = vz;
      reinterpret_cast<float4*>(mvel)[m] = mv;
      st_f4(st_out, 2 * p, make_float4(0.f, 0.f, 0.f, __uint_as_float(SLOT_EMPTY)));
      st_f4(st_out, 2 * p + 1, make_float4(0.f, 0.f, 0.f, 0.f));
    } else {
      // final image c_t of the streamed point; the velocity already carries -c_s
      float ys = __fadd_rn(x.y, f.shift[1]);
      float X = x.x, Y = x.y, Z = x.z;
      if (fabsf(X) < 1.5f * f.L[0] && fabsf(ys) < 1.5f * f.L[1] && fabsf(Y) < 1.5f * f.L[1] &&
          fabsf(Z) < 1.5f * f.L[2]) {
        // every streamed point in practice: selects only
        if (f.shear_on) {
          const float cs = img_sel(ys, f.half[1]);
          const float ct = img_sel(Y, f.half[1]);
          Y = fmaf(-ct, f.L[1], Y);
          X = wrap_sel(fmaf(-ct, f.delrx, X), f.L[0], f.half[0]);
          vx = fmaf(-(ct - cs), f.shearLy, vx);
        } else {
          X = wrap_sel(X, f.L[0], f.half[0]);
          Y = wrap_sel(Y, f.L[1], f.half[1]);
        }
        Z = wrap_sel(Z, f.L[2], f.half[2]);
        st_f4(st_out, 2 * p, make_float4(X, Y, Z, x.w));
        st_f4(st_out, 2 * p + 1, make_float4(vx, vy, vz, 0.f));
        continue;
      }
      const float cs = f.shear_on ? img_f(ys, f.L[1], f.half[1]) : 0.0f;
      if (f.shear_on) {
        const float ct = img_f(Y, f.L[1], f.half[1]);
        Y = __fsub_rn(Y, __fmul_rn(ct, f.L[1]));
        X = wrap_f(__fsub_rn(X, __fmul_rn(ct, f.delrx)), f.L[0], f.half[0]);
        vx = __fsub_rn(vx, __fmul_rn(ct - cs, f.shearLy));
      } else {
        X = wrap_f(X, f.L[0], f.half[0]);
        Y = wrap_f(Y, f.L[1], f.half[1]);
      }
      Z = wrap_f(Z, f.L[2], f.half[2]);
      st_f4(st_out, 2 * p, make_float4(X, Y, Z, x.w));
      st_f4(st_out, 2 * p + 1, make_float4(vx, vy, vz, 0.f));
    }
  }
}

template <int NT, int CT, int CAP, int GU>
__global__ void __launch_bounds__(NT) k_collide_f32(
    const Tile* tiles, const RepInfo* reps, const FrameF* frames, const RepDyn* dyn,
    const uint32_t* __restrict__ off, const uint32_t* __restrict__ perm,
    const float* __restrict__ st_in, float* __restrict__ st_out, const float* mpos, float* mvel,
    const int* mimg, const double* inj_gamma, const double* inj_uphi, const double* inj_utheta,
    int rng, int mono_bin, ErrorState* err) {
  static_assert(NT == 2 * CT, "two threads per cell");
  __shared__ float4 s_rc[CT * 3];  // per cell: rows of sR, cell velocity in .w
  __shared__ uint32_t s_off[CT + 1];
  extern __shared__ __align__(16) unsigned char s_dyn[];
  float4* s_x = reinterpret_cast<float4*>(s_dyn);
  float4* s_v = s_x + CAP;
  short* s_lc = reinterpret_cast<short*>(s_v + CAP);

  const Tile t = tiles[blockIdx.x];
  const FrameF f = frames[t.rep];
  const RepInfo& ri = reps[t.rep];
  const unsigned long long seed = ri.seed;
  const unsigned long long step = dyn[t.rep].step;
  const uint32_t cbase = static_cast<uint32_t>(ri.cell_base);
  const int nc = t.end - t.begin;

  for (int i = threadIdx.x; i <= nc; i += NT) s_off[i] = off[t.begin + i];
  __syncthreads();
  const uint32_t p0 = s_off[0], p1 = s_off[nc];
  const int n = static_cast<int>(p1 - p0);
  const int nloc = n < CAP ? n : CAP;

  // stage: gather, stream, collision-frame velocity
  for (int base = 0; base < nloc; base += NT * GU) {
    uint32_t src[GU];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int j = base + u * NT + threadIdx.x;
      src[u] = j < nloc ? perm[p0 + j] : 0u;
    }
    FastP P[GU];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int j = base + u * NT + threadIdx.x;
      if (j < nloc) fetch_f(P[u], src[u], st_in, mpos, mvel, mimg, f, mono_bin);
    }
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int j = base + u * NT + threadIdx.x;
      if (j < nloc) {
        frame_f(P[u], f, f.solvent_mass);
        s_x[j] = P[u].x;
        s_v[j] = P[u].v;
      }
    }
  }
  __syncthreads();

  const CollideF32Args A{st_in, st_out, mpos, mvel, mimg, perm, inj_gamma, inj_uphi, inj_utheta,
                         rng, mono_bin, err};
  collide_cells_f32<NT>(A, f, t, s_off, nc, p0, nloc, s_x, s_v, s_lc, s_rc, seed, step,
                        cbase);
  __syncthreads();
  collide_apply_f32<NT>(A, f, s_off, p0, n, nloc, s_x, s_v, s_lc, s_rc);
}

// ------------------------------------------------- collide, cp.async staging
// k_collide_f32 with the gather done by cp.async: every thread first loads
// the sorted slots of all its staged particles, then issues all their 16-byte
// record copies straight into shared memory (no registers hold data in
// flight), then the streaming / collision-frame pass runs in place. A tile
// costs three dependent load rounds (offsets, slots, records) whatever its
// size, with the shared memory and register budget of k_collide_f32. The
// arithmetic is the same as k_collide_f32's, so both give identical bits.

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

template <int NT, int CT, int CAP>
__global__ void __launch_bounds__(NT) k_collide_f32_async(
    const Tile* tiles, const RepInfo* reps, const FrameF* frames, const RepDyn* dyn,
    const uint32_t* __restrict__ off, const uint32_t* __restrict__ perm,
    const float* __restrict__ st_in, float* __restrict__ st_out, const float* mpos, float* mvel,
    const int* mimg, const double* inj_gamma, const double* inj_uphi, const double* inj_utheta,
    int rng, int mono_bin, ErrorState* err) {
  // two threads per cell in the cell pass; threads past 2 CT take no cell
  // there and add warps to the particle passes (gather, frame, apply)
  static_assert(NT >= 2 * CT && NT % 32 == 0, "two threads per cell, whole warps");
  constexpr int J = (CAP + NT - 1) / NT;  // staged particles per thread
  __shared__ float4 s_rc[CT * 3];  // per cell: rows of sR, cell velocity in .w
  __shared__ uint32_t s_off[CT + 1];
  extern __shared__ __align__(16) unsigned char s_dyn[];
  float4* s_x = reinterpret_cast<float4*>(s_dyn);
  float4* s_v = s_x + CAP;
  short* s_lc = reinterpret_cast<short*>(s_v + CAP);

  const Tile t = tiles[blockIdx.x];
  const int nc = t.end - t.begin;
  for (int i = threadIdx.x; i <= nc; i += NT) s_off[i] = off[t.begin + i];
  __syncthreads();
  const uint32_t p0 = s_off[0];
  const int n = static_cast<int>(s_off[nc] - p0);
  const int nloc = n < CAP ? n : CAP;

  uint32_t src[J];
#pragma unroll
  for (int u = 0; u < J; ++u) {
    const int j = u * NT + threadIdx.x;
    src[u] = j < nloc ? perm[p0 + j] : 0xFFFFFFFFu;
  }
#pragma unroll
  for (int u = 0; u < J; ++u) {
    const int j = u * NT + threadIdx.x;
    if (src[u] != 0xFFFFFFFFu) {
      if (src[u] & MONO_BIT) {
        cp_async16(s_v + j, mvel + 4 * static_cast<size_t>(src[u] & ~MONO_BIT));
        s_x[j] = make_float4(0.f, 0.f, 0.f, __uint_as_float(src[u]));
      } else {
        cp_async16(s_x + j, st_in + 8 * static_cast<size_t>(src[u]));
        cp_async16(s_v + j, st_in + 8 * static_cast<size_t>(src[u]) + 4);
      }
    }
  }
  const FrameF f = frames[t.rep];
  const RepInfo& ri = reps[t.rep];
  cp_async_wait_all();
  // each thread finishes the particles it copied: stream and move into the
  // collision frame, in place (fetch_f + frame_f)
#pragma unroll
  for (int u = 0; u < J; ++u) {
    const int j = u * NT + threadIdx.x;
    if (src[u] == 0xFFFFFFFFu) break;  // this thread's remaining slots are past nloc too
    FastP P;
    P.x = s_x[j];
    P.v = s_v[j];
    if (src[u] & MONO_BIT) {
      const uint32_t m = src[u] & ~MONO_BIT;
      P.v.w = reinterpret_cast<const float4*>(mpos)[m].w;
      if (mono_bin == MONOBIN_WRAPPED)
        P.v.x = __fsub_rn(P.v.x, __fmul_rn(i2f_small(mimg[m]), f.shearLy));
    } else {
      frame_f(P, f, f.solvent_mass);
    }
    s_x[j] = P.x;
    s_v[j] = P.v;
  }
  __syncthreads();

  const CollideF32Args A{st_in, st_out, mpos, mvel, mimg, perm, inj_gamma, inj_uphi, inj_utheta,
                         rng, mono_bin, err};
  collide_cells_f32<NT>(A, f, t, s_off, nc, p0, nloc, s_x, s_v, s_lc, s_rc, ri.seed,
                        dyn[t.rep].step, static_cast<uint32_t>(ri.cell_base));
  __syncthreads();
  collide_apply_f32<NT>(A, f, s_off, p0, n, nloc, s_x, s_v, s_lc, s_rc);
}

}  // namespace smpc
