// MPC (SRD) collision-step kernels, templated on the storage/arithmetic type
// R (double for the FP64 reference-parity path, float for the fast path).
//
// One collision (MPC::step, star-polymers/lib/Hydrodynamics/MPC.cpp:116-142):
//   k_cycle_begin  delrx advance (MPC.cpp:117-118) + Philox grid shift   [graph mode]
//   k_mono_prep    check_bounds recentring (MPC.cpp:160-190), monomer grid shift
//                  (MPC.cpp:306-310) and monomer binning (MPC.cpp:221-236)
//   k_fluid_bin    recentre/stream/shift/LE-wrap each solvent particle
//                  (MPC.cpp:183-197, 301-305, 421-429) and bin it: cell key and
//                  rank from one warp-aggregated atomic per (warp, cell)
//   scan           exclusive prefix of the cell counts (scan.cu)
//   k_build_perm   counting-sort scatter: sorted position -> source
//   k_collide      per tile of cells: gathers its particles into shared memory,
//                  recomputes their streamed/shifted state, reduces per-cell
//                  momentum, mass and kinetic energy (one thread per cell over
//                  the staged particles; int64 fixed point on the fast path),
//                  draws the MBS thermostat and the rotation (MPC.cpp:239-299),
//                  applies them, undoes the shift (MPC.cpp:139-140) and writes
//                  the solvent back in cell order (next step's input is sorted).
#pragma once
#include <stdint.h>

#include <type_traits>

#include "philox.cuh"
#include "smpc_device.cuh"

namespace smpc {

// ------------------------------------------------------------ load / store

template <typename R>
struct R4 {
  R x, y, z, w;
};

__device__ __forceinline__ R4<float> ld4(const float* p, size_t i) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p) + i);
  return R4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ R4<double> ld4(const double* p, size_t i) {
  const double2* q = reinterpret_cast<const double2*>(p) + 2 * i;
  const double2 a = __ldg(q), b = __ldg(q + 1);
  return R4<double>{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ R4<float> ld4_rw(const float* p, size_t i) {
  const float4 v = reinterpret_cast<const float4*>(p)[i];
  return R4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ R4<double> ld4_rw(const double* p, size_t i) {
  const double2* q = reinterpret_cast<const double2*>(p) + 2 * i;
  const double2 a = q[0], b = q[1];
  return R4<double>{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st4(float* p, size_t i, const R4<float>& v) {
  reinterpret_cast<float4*>(p)[i] = make_float4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ void st4(double* p, size_t i, const R4<double>& v) {
  double2* q = reinterpret_cast<double2*>(p) + 2 * i;
  q[0] = make_double2(v.x, v.y);
  q[1] = make_double2(v.z, v.w);
}

// Solvent slot records: position then velocity of slot i are adjacent
// (8 Reals, 32 B in FP32), so a gathered particle is one 32-byte sector.
template <typename R>
__device__ __forceinline__ R4<R> ld_pos(const R* st, size_t i) { return ld4(st, 2 * i); }
template <typename R>
__device__ __forceinline__ R4<R> ld_vel(const R* st, size_t i) { return ld4(st, 2 * i + 1); }
template <typename R>
__device__ __forceinline__ void st_rec(R* st, size_t i, const R4<R>& x, const R4<R>& v) {
  st4(st, 2 * i, x);
  st4(st, 2 * i + 1, v);
}

// The slot's id travels in the .w word as a bit pattern, never as a number:
// FP32 the word itself, FP64 the low half of the double (a zero or subnormal
// value that no arithmetic ever reads). Reading it is an integer move, not a
// conversion, which on GB300 would issue on the narrow FP64 pipe.
__device__ __forceinline__ uint32_t slot_id(float w) { return __float_as_uint(w); }
__device__ __forceinline__ uint32_t slot_id(double w) {
  return static_cast<uint32_t>(__double_as_longlong(w));
}
template <typename R>
__device__ __forceinline__ R make_slot_id(uint32_t id);
template <>
__device__ __forceinline__ float make_slot_id<float>(uint32_t id) { return __uint_as_float(id); }
template <>
__device__ __forceinline__ double make_slot_id<double>(uint32_t id) {
  return __longlong_as_double(static_cast<long long>(id));
}

// ------------------------------------------------------- box geometry

// Explicitly rounded arithmetic for the particle frame transform. These are
// never contracted into FMAs, so k_fluid_bin and k_collide (which recomputes
// the transform) produce bit-identical coordinates and cell keys in both
// precisions, whatever the surrounding code is optimised into.
__device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float r_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double r_div(double a, double b) { return __ddiv_rn(a, b); }

// Per-replica constants in the working precision. The FP64 path follows the
// reference's operation order exactly (-fmad=false): round-half-away,
// division by L, (cy*shear)*Ly. The FP32 path uses the same operations.
// Everything is converted to R once per thread block, so the FP32 hot loops
// never touch the (slow on GB300) FP64 pipe.
template <typename R>
struct Geo {
  R L[3];
  R half[3];
  int Li[3];
  R shear;
  R delrx;
  bool shear_on;
  int wrap_mono;
  // this collision's frame: grid shift, streaming time, recentring
  R shift[3];
  R com[3];
  R comv[3];
  R h;
  bool recentre;
  // FP64 wraps (le_wrap<double>): bit patterns of L/2 (1 - 2^-50), L/2 and
  // 1.5 L (1 - 2^-50) per axis
  long long w_lo[3], w_half[3], w_far[3];
};

template <typename R>
__device__ __forceinline__ Geo<R> make_geo(const RepInfo& ri, const RepDyn& dn, int mono_bin) {
  Geo<R> g;
  for (int d = 0; d < 3; ++d) {
    g.L[d] = static_cast<R>(ri.L[d]);
    g.half[d] = static_cast<R>(ri.L[d]) * R(0.5);
    g.Li[d] = ri.L[d];
    g.shift[d] = static_cast<R>(dn.shift[d]);
    g.com[d] = static_cast<R>(dn.com[d]);
    g.comv[d] = static_cast<R>(dn.comv[d]);
  }
  g.shear = static_cast<R>(ri.shear);
  g.delrx = static_cast<R>(dn.delrx);
  g.shear_on = (ri.shear != 0.0);
  g.wrap_mono = mono_bin;
  g.h = static_cast<R>(dn.h);
  g.recentre = dn.recentre != 0;
  for (int d = 0; d < 3; ++d) {
    const double half = static_cast<double>(ri.L[d]) * 0.5;
    g.w_lo[d] = __double_as_longlong(half * (1.0 - 0x1.0p-50));
    g.w_half[d] = __double_as_longlong(half);
    g.w_far[d] = __double_as_longlong(3.0 * half * (1.0 - 0x1.0p-50));
  }
  return g;
}

// MPC::wrap(Particle&) -> LEBC (MPC.cpp:421-429) or periodic wrap (MPC.cpp:473-478).
template <typename R>
__device__ __forceinline__ void le_wrap(const Geo<R>& g, R& x, R& y, R& z, R& vx) {
  if (g.shear_on) {
    const R cy = r_round(r_div(y, g.L[1]));
    x = r_sub(x, r_mul(g.L[0], r_round(r_div(x, g.L[0]))));
    x = r_sub(x, r_mul(cy, g.delrx));
    x = r_sub(x, r_mul(g.L[0], r_round(r_div(x, g.L[0]))));
    y = r_sub(y, r_mul(g.L[1], cy));
    z = r_sub(z, r_mul(g.L[2], r_round(r_div(z, g.L[2]))));
    vx = r_sub(vx, r_mul(r_mul(cy, g.shear), g.L[1]));
  } else {
    x = r_sub(x, r_mul(r_round(r_div(x, g.L[0])), g.L[0]));
    y = r_sub(y, r_mul(r_round(r_div(y, g.L[1])), g.L[1]));
    z = r_sub(z, r_mul(r_round(r_div(z, g.L[2])), g.L[2]));
  }
}

// FP64: the same results as the formula above, bit for bit (signed zeros
// aside), without its divisions and roundings, which on this part run on the
// narrow FP64 pipe (2 instructions per clock per SM) and made the FP64 solvent
// kernels FP64-bound. round(x / L) is decided from the magnitude bits of x,
// whose integer order is the order of non-negative doubles: it is 0 below
// L/2 (1 - 2^-50) and +-1 from L/2 (x / L >= 1/2 rounds away from zero) up
// to 1.5 L (1 - 2^-50); in the two narrow bands in between, where rounding
// x / L can reach 1/2 or 3/2, and beyond, the formula itself decides. x - L
// and x + L are the formula's x - L round(x / L) for round = +-1 exactly.
__device__ __forceinline__ double image_d(double y, double L, long long lo, long long half,
                                          long long far) {
  const long long bits = __double_as_longlong(y);
  const long long ax = bits & 0x7FFFFFFFFFFFFFFFll;
  if (ax < lo) return 0.0;
  if (ax >= half && ax < far) return bits < 0 ? -1.0 : 1.0;
  return r_round(r_div(y, L));
}
__device__ __forceinline__ double wrap_d(double x, double L, long long lo, long long half,
                                         long long far) {
  const long long bits = __double_as_longlong(x);
  const long long ax = bits & 0x7FFFFFFFFFFFFFFFll;
  if (ax < lo) return x;
  if (ax >= half && ax < far) return bits < 0 ? r_add(x, L) : r_sub(x, L);
  return r_sub(x, r_mul(L, r_round(r_div(x, L))));
}
// The general case of le_wrap<double>, out of line: called only when a
// coordinate is at or past L/2 (1 - 2^-50), so that its FP64 instructions run
// for those particles only (inlined, the compiler predicates its short
// branches and every warp issues them on the FP64 pipe). Everything goes by
// value, so no caller's state has to live in memory.
struct WrapD {
  double x, y, z, vx;
};
struct WrapConstD {
  double L[3];
  long long lo[3], half[3], far[3];
  double delrx, shear;
  int shear_on;
};
static __device__ __noinline__ WrapD le_wrap_d_general(WrapD p, WrapConstD c) {
  if (c.shear_on) {
    const double cy = image_d(p.y, c.L[1], c.lo[1], c.half[1], c.far[1]);
    p.x = wrap_d(p.x, c.L[0], c.lo[0], c.half[0], c.far[0]);
    if (cy != 0.0) p.x = r_sub(p.x, r_mul(cy, c.delrx));
    p.x = wrap_d(p.x, c.L[0], c.lo[0], c.half[0], c.far[0]);
    if (cy != 0.0) {
      p.y = r_sub(p.y, r_mul(c.L[1], cy));
      p.vx = r_sub(p.vx, r_mul(r_mul(cy, c.shear), c.L[1]));
    }
    p.z = wrap_d(p.z, c.L[2], c.lo[2], c.half[2], c.far[2]);
  } else {
    p.x = wrap_d(p.x, c.L[0], c.lo[0], c.half[0], c.far[0]);
    p.y = wrap_d(p.y, c.L[1], c.lo[1], c.half[1], c.far[1]);
    p.z = wrap_d(p.z, c.L[2], c.lo[2], c.half[2], c.far[2]);
  }
  return p;
}
template <>
__device__ __forceinline__ void le_wrap<double>(const Geo<double>& g, double& x, double& y,
                                                double& z, double& vx) {
  // below L/2 (1 - 2^-50) on every axis the formula changes nothing: no
  // image in y, and every wrap_d returns its argument
  const long long ax = __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFll;
  const long long ay = __double_as_longlong(y) & 0x7FFFFFFFFFFFFFFFll;
  const long long az = __double_as_longlong(z) & 0x7FFFFFFFFFFFFFFFll;
  if (ax < g.w_lo[0] && ay < g.w_lo[1] && az < g.w_lo[2]) return;
  WrapConstD c;
  for (int d = 0; d < 3; ++d) {
    c.L[d] = g.L[d];
    c.lo[d] = g.w_lo[d];
    c.half[d] = g.w_half[d];
    c.far[d] = g.w_far[d];
  }
  c.delrx = g.delrx;
  c.shear = g.shear;
  c.shear_on = g.shear_on ? 1 : 0;
  const WrapD r = le_wrap_d_general(WrapD{x, y, z, vx}, c);
  x = r.x;
  y = r.y;
  z = r.z;
  vx = r.vx;
}

// FP32 fast path: one conditional image shift per axis, exact (x - L is
// exact for x in [L/2, 2L]) and free of division and rounding. Valid while
// every coordinate is within 1.5 L of the origin, which one streaming step
// (|v| h < L) and one grid shift keep true; otherwise the general formula.
// Coordinates exactly at -L/2 stay at -L/2 (the general formula maps them to
// +L/2); both are the same face of the periodic box.
__device__ __forceinline__ float wrap1f(float x, float L, float half) {
  return x >= half ? r_sub(x, L) : (x < -half ? r_add(x, L) : x);
}
__device__ __forceinline__ void le_wrap(const Geo<float>& g, float& x, float& y, float& z,
                                        float& vx) {
  if (!(fabsf(x) < 1.5f * g.L[0] && fabsf(y) < 1.5f * g.L[1] && fabsf(z) < 1.5f * g.L[2])) {
    le_wrap<float>(g, x, y, z, vx);
    return;
  }
  if (g.shear_on) {
    const float cy = y >= g.half[1] ? 1.0f : (y < -g.half[1] ? -1.0f : 0.0f);
    x = wrap1f(x, g.L[0], g.half[0]);
    x = r_sub(x, r_mul(cy, g.delrx));
    x = wrap1f(x, g.L[0], g.half[0]);
    y = r_sub(y, r_mul(g.L[1], cy));
    z = wrap1f(z, g.L[2], g.half[2]);
    vx = r_sub(vx, r_mul(r_mul(cy, g.shear), g.L[1]));
  } else {
    x = wrap1f(x, g.L[0], g.half[0]);
    y = wrap1f(y, g.L[1], g.half[1]);
    z = wrap1f(z, g.L[2], g.half[2]);
  }
}

// Cell index of MPC::sort (MPC.cpp:209). strict: the reference's formula,
// aliasing included, range-checked only against the last cell like the
// reference; otherwise every axis index is clamped into the box (the fast
// path: positions exactly on the upper face round onto L in FP32).
template <typename R>
__device__ __forceinline__ uint32_t cell_of(const Geo<R>& g, R x, R y, R z, bool strict) {
  int ix = static_cast<int>(r_add(x, g.half[0]));
  int iy = static_cast<int>(r_add(y, g.half[1]));
  int iz = static_cast<int>(r_add(z, g.half[2]));
  if (strict) {
    const int c = ix + g.Li[0] * iy + g.Li[0] * g.Li[1] * iz;
    return static_cast<uint32_t>(c);
  }
  ix = min(max(ix, 0), g.Li[0] - 1);
  iy = min(max(iy, 0), g.Li[1] - 1);
  iz = min(max(iz, 0), g.Li[2] - 1);
  return static_cast<uint32_t>(ix + g.Li[0] * (iy + g.Li[1] * iz));
}

// FP32 fast path (never strict): floor by directed-rounding add, clamped.
__device__ __forceinline__ uint32_t cell_of(const Geo<float>& g, float x, float y, float z,
                                            bool strict) {
  if (strict) return cell_of<float>(g, x, y, z, true);
  const int ix = min(f2i_floor_nonneg(fmaxf(r_add(x, g.half[0]), 0.0f)), g.Li[0] - 1);
  const int iy = min(f2i_floor_nonneg(fmaxf(r_add(y, g.half[1]), 0.0f)), g.Li[1] - 1);
  const int iz = min(f2i_floor_nonneg(fmaxf(r_add(z, g.half[2]), 0.0f)), g.Li[2] - 1);
  return static_cast<uint32_t>(ix + g.Li[0] * (iy + g.Li[1] * iz));
}

__device__ __forceinline__ void raise_error(ErrorState* e, uint32_t bit, uint32_t a, uint32_t b) {
  const uint32_t old = atomicOr(&e->word, bit);
  if ((old & bit) == 0) {
    e->info[0] = bit;
    e->info[1] = a;
    e->info[2] = b;
  }
}

// Solvent particle from its stored state to the shifted collision frame:
// [recentre: x -= COM, v -= COMV, wrap] -> stream x += v h, wrap -> x += s, wrap.
template <typename R>
__device__ __forceinline__ void fluid_to_collision_frame(const Geo<R>& g, R4<R>& x, R4<R>& v) {
  if (g.recentre) {
    x.x = r_sub(x.x, g.com[0]);
    x.y = r_sub(x.y, g.com[1]);
    x.z = r_sub(x.z, g.com[2]);
    v.x = r_sub(v.x, g.comv[0]);
    v.y = r_sub(v.y, g.comv[1]);
    v.z = r_sub(v.z, g.comv[2]);
    le_wrap(g, x.x, x.y, x.z, v.x);
  }
  x.x = r_add(x.x, r_mul(v.x, g.h));
  x.y = r_add(x.y, r_mul(v.y, g.h));
  x.z = r_add(x.z, r_mul(v.z, g.h));
  le_wrap(g, x.x, x.y, x.z, v.x);
  x.x = r_add(x.x, g.shift[0]);
  x.y = r_add(x.y, g.shift[1]);
  x.z = r_add(x.z, g.shift[2]);
  le_wrap(g, x.x, x.y, x.z, v.x);
}

// Warp-aggregated rank: one atomicAdd per distinct key in the warp. All 32
// lanes must call it (key KEY_NONE for idle lanes).
__device__ __forceinline__ uint32_t warp_rank(uint32_t* count, uint32_t key) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (static_cast<int>(lane) == leader && key != KEY_NONE) base = atomicAdd(count + key, __popc(peers));
  base = __shfl_sync(0xFFFFFFFFu, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

// ------------------------------------------------------------ kernels

// Graph mode: advance delrx n_sub times exactly as MPC.cpp:117-118 does on
// every MD step, draw this collision's grid shift from Philox, and latch the
// collision counter. One thread per replica.
template <typename R>
__global__ void k_cycle_begin(const RepInfo* reps, RepDyn* dyn, int n_rep, int n_adv,
                              double adv_scale, int gen_shift) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rep) return;
  const RepInfo ri = reps[r];
  RepDyn& dn = dyn[r];
  double d = dn.delrx;
  const double Lx = static_cast<double>(ri.L[0]);
  const double adv_dt = __dmul_rn(ri.h, adv_scale);
  if (n_adv > 0) dn.h = ri.h;
  for (int s = 0; s < n_adv; ++s) {
    d = __dadd_rn(d, __dmul_rn(__dmul_rn(ri.shear, static_cast<double>(ri.L[1])), adv_dt));
    d = __dsub_rn(d, __dmul_rn(Lx, round(__ddiv_rn(d, Lx))));
  }
  dn.delrx = d;
  if (gen_shift) {
    const unsigned long long step = dn.step;
    const Uniform2<double> a = philox_uniforms<double>(ri.seed, 0xFFFFFFFFu, step, 0u);
    const Uniform2<double> b = philox_uniforms<double>(ri.seed, 0xFFFFFFFFu, step, 1u);
    dn.shift[0] = a.a - 0.5;
    dn.shift[1] = a.b - 0.5;
    dn.shift[2] = b.a - 0.5;
  }
}

template <typename R>
__global__ void k_cycle_end(RepDyn* dyn, int n_rep) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n_rep) dyn[r].step += 1ull;
}

// Solvent initial state on the device for one replica: positions uniform in
// the box, velocities Maxwell-Boltzmann at kT (or, with ref_vel, uniform in
// [-1/2, 1/2) as MPC::initialize draws them, MPC.cpp:37-41; the mean is not
// removed here). Counter-based: particle i of replica seed s always gets the
// same values. Slots past n_fluid become holes.
template <typename R>
__global__ void k_init_solvent(const RepInfo* reps, int rep, R* st, unsigned long long seed,
                               double kT, int flags) {
  const int ref_vel = flags & 1;  // smpc.h SMPC_INIT_REFERENCE_VELOCITIES
  const RepInfo ri = reps[rep];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ri.slot_cap) return;
  const size_t slot = static_cast<size_t>(ri.slot_base) + i;
  if (i >= ri.n_fluid) {
    st_rec(st, slot, R4<R>{R(0), R(0), R(0), make_slot_id<R>(SLOT_EMPTY)},
           R4<R>{R(0), R(0), R(0), R(0)});
    return;
  }
  const Uniform2<double> a = philox_uniforms<double>(seed, static_cast<uint32_t>(i), 0xA11CEull, 0u);
  const Uniform2<double> b = philox_uniforms<double>(seed, static_cast<uint32_t>(i), 0xA11CEull, 1u);
  const Uniform2<double> c = philox_uniforms<double>(seed, static_cast<uint32_t>(i), 0xA11CEull, 2u);
  const Uniform2<double> d = philox_uniforms<double>(seed, static_cast<uint32_t>(i), 0xA11CEull, 3u);
  R4<R> x{static_cast<R>((a.a - 0.5) * ri.L[0]), static_cast<R>((a.b - 0.5) * ri.L[1]),
          static_cast<R>((b.a - 0.5) * ri.L[2]), make_slot_id<R>(static_cast<uint32_t>(i))};
  R4<R> v;
  if (ref_vel) {
    v = R4<R>{static_cast<R>(b.b - 0.5), static_cast<R>(c.a - 0.5), static_cast<R>(c.b - 0.5), R(0)};
  } else {
    const double sd = sqrt(kT / ri.solvent_mass);
    const double r1 = sqrt(-2.0 * log(b.b)), r2 = sqrt(-2.0 * log(c.b));
    const double t1 = 6.283185307179586 * c.a, t2 = 6.283185307179586 * d.a;
    v = R4<R>{static_cast<R>(sd * r1 * cos(t1)), static_cast<R>(sd * r1 * sin(t1)),
              static_cast<R>(sd * r2 * cos(t2)), R(0)};
  }
  st_rec(st, slot, x, v);
}

// MPC::initialize removes the mean of the drawn velocities (MPC.cpp:42-48).
// k_init_velocity_sum: per-block FP64 sums over the replica's solvent with a
// fixed grid (grid-stride, warp butterflies, warps joined in order), so the
// mean does not depend on scheduling. k_init_velocity_finish: every thread
// sums the block partials in order, subtracts the mean, then adds the steady
// flow shear * y to v_x for SMPC_INIT_SHEAR_PROFILE.
constexpr int INIT_SUM_BLOCKS = 256;
constexpr int INIT_SUM_THREADS = 256;

template <typename R>
__global__ void __launch_bounds__(INIT_SUM_THREADS)
    k_init_velocity_sum(const RepInfo* reps, int rep, const R* st, double* part) {
  const RepInfo ri = reps[rep];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * INIT_SUM_THREADS + threadIdx.x; i < ri.n_fluid;
       i += INIT_SUM_BLOCKS * INIT_SUM_THREADS) {
    const R4<R> v = ld_vel(st, static_cast<size_t>(ri.slot_base) + i);
    s0 += static_cast<double>(v.x);
    s1 += static_cast<double>(v.y);
    s2 += static_cast<double>(v.z);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xFFFFFFFFu, s0, o);
    s1 += __shfl_xor_sync(0xFFFFFFFFu, s1, o);
    s2 += __shfl_xor_sync(0xFFFFFFFFu, s2, o);
  }
  __shared__ double w[INIT_SUM_THREADS / 32][3];
  if ((threadIdx.x & 31) == 0) {
    w[threadIdx.x >> 5][0] = s0;
    w[threadIdx.x >> 5][1] = s1;
    w[threadIdx.x >> 5][2] = s2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int k = 0; k < INIT_SUM_THREADS / 32; ++k) t += w[k][threadIdx.x];
    part[3 * blockIdx.x + threadIdx.x] = t;
  }
}

template <typename R>
__global__ void k_init_velocity_finish(const RepInfo* reps, int rep, R* st, const double* part,
                                       int flags) {
  const RepInfo ri = reps[rep];
  __shared__ double s_mean[3];
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int b = 0; b < INIT_SUM_BLOCKS; ++b) t += part[3 * b + threadIdx.x];
    s_mean[threadIdx.x] = ri.n_fluid > 0 ? t / static_cast<double>(ri.n_fluid) : 0.0;
  }
  __syncthreads();
  const double m0 = s_mean[0], m1 = s_mean[1], m2 = s_mean[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ri.n_fluid;
       i += gridDim.x * blockDim.x) {
    const size_t slot = static_cast<size_t>(ri.slot_base) + i;
    const R4<R> x = ld_pos(st, slot);
    R4<R> v = ld_vel(st, slot);
    double vx = static_cast<double>(v.x) - m0;
    if (flags & 2)  // SMPC_INIT_SHEAR_PROFILE: the steady flow shear * y
      vx += ri.shear * static_cast<double>(x.y);
    v.x = static_cast<R>(vx);
    v.y = static_cast<R>(static_cast<double>(v.y) - m1);
    v.z = static_cast<R>(static_cast<double>(v.z) - m2);
    st4(st, 2 * slot + 1, v);
  }
}

// One CTA per replica: MPC::check_bounds, then shift and bin the monomers.
// A replica that cannot recentre (mol0_size == 0, e.g. a periodic box) has
// independent monomers: it is split over the gridDim.y CTAs of its row.
template <typename R, int NT>
__global__ void __launch_bounds__(NT) k_mono_prep(const RepInfo* reps, RepDyn* dyn, R* mpos,
                                                  R* mvel, uint2* mkey, int* mimg,
                                                  uint32_t* count, ErrorState* err,
                                                  int mono_bin, int strict, FrameF* frames,
                                                  double rot_c, double rot_s) {
  const int r = blockIdx.x;
  const RepInfo ri = reps[r];
  const bool split = ri.mol0_size == 0;
  if (blockIdx.y > 0 && !split) return;
  __shared__ int s_out;
  if (threadIdx.x == 0) s_out = 0;
  __syncthreads();
  const int per = split ? (ri.n_mono + gridDim.y - 1) / gridDim.y : ri.n_mono;
  const int b = ri.mono_base + static_cast<int>(blockIdx.y) * per;
  const int n = max(0, min(per, ri.n_mono - static_cast<int>(blockIdx.y) * per));
  // MPC.cpp:166: any monomer with |x_d| >= L_d/2 - 0.5 triggers recentring
  for (int i = threadIdx.x; i < n && !split; i += NT) {
    const R4<R> x = ld4_rw(mpos, b + i);
    const R xs[3] = {x.x, x.y, x.z};
    for (int d = 0; d < 3; ++d)
      if (r_fabs(xs[d]) >= (static_cast<R>(ri.L[d]) * R(0.5) - R(0.5))) s_out = 1;
  }
  __syncthreads();
  RepDyn& dn = dyn[r];
  const int out = s_out && ri.mol0_size > 0;
  if (!std::is_same<R, double>::value && out) {
    // fast path: block-parallel centre of mass (FP64 sums, order free)
    __shared__ double s_c[6];
    if (threadIdx.x < 6) s_c[threadIdx.x] = 0.0;
    __syncthreads();
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < ri.mol0_size; i += NT) {
      const R4<R> x = ld4_rw(mpos, b + i);
      const R4<R> v = ld4_rw(mvel, b + i);
      c[0] += x.x; c[1] += x.y; c[2] += x.z;
      c[3] += v.x; c[4] += v.y; c[5] += v.z;
    }
    for (int q = 0; q < 6; ++q) {
      double t = c[q];
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
      if ((threadIdx.x & 31) == 0) atomicAdd(&s_c[q], t);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      dn.recentre = 1;
      const double nm = static_cast<double>(ri.mol0_size);
      for (int d = 0; d < 3; ++d) {
        dn.com[d] = s_c[d] / nm;
        dn.comv[d] = s_c[3 + d] / nm;
      }
    }
  } else if (threadIdx.x == 0 && blockIdx.y == 0) {
    dn.recentre = out;
    if (out) {
      // Molecule::calculate_center_of_mass[_velocity] (Molecule.cpp:139-155):
      // sequential sums over molecule 0, as the reference does.
      double c[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
      for (int i = 0; i < ri.mol0_size; ++i) {
        const R4<R> x = ld4_rw(mpos, b + i);
        const R4<R> v = ld4_rw(mvel, b + i);
        c[0] = __dadd_rn(c[0], static_cast<double>(x.x));
        c[1] = __dadd_rn(c[1], static_cast<double>(x.y));
        c[2] = __dadd_rn(c[2], static_cast<double>(x.z));
        cv[0] = __dadd_rn(cv[0], static_cast<double>(v.x));
        cv[1] = __dadd_rn(cv[1], static_cast<double>(v.y));
        cv[2] = __dadd_rn(cv[2], static_cast<double>(v.z));
      }
      const double nm = static_cast<double>(static_cast<unsigned>(ri.mol0_size));
      for (int d = 0; d < 3; ++d) {
        dn.com[d] = __ddiv_rn(c[d], nm);
        dn.comv[d] = __ddiv_rn(cv[d], nm);
      }
    }
  }
  __syncthreads();
  const Geo<R> g = make_geo<R>(ri, dn, mono_bin);
  const R s0 = static_cast<R>(dn.shift[0]), s1 = static_cast<R>(dn.shift[1]),
          s2 = static_cast<R>(dn.shift[2]);
  const R c0 = static_cast<R>(dn.com[0]), c1 = static_cast<R>(dn.com[1]),
          c2 = static_cast<R>(dn.com[2]);
  const R cv0 = static_cast<R>(dn.comv[0]), cv1 = static_cast<R>(dn.comv[1]),
          cv2 = static_cast<R>(dn.comv[2]);
  const int iters = (n + NT - 1) / NT;
  for (int it = 0; it < iters; ++it) {
    const int i = it * NT + threadIdx.x;
    uint32_t key = KEY_NONE;
    R4<R> x{}, v{};
    int img = 0;
    if (i < n) {
      x = ld4_rw(mpos, b + i);
      v = ld4_rw(mvel, b + i);
      if (out) {
        x.x -= c0; x.y -= c1; x.z -= c2;
        v.x -= cv0; v.y -= cv1; v.z -= cv2;
        st4(mvel, b + i, v);
      }
      x.x += s0; x.y += s1; x.z += s2;  // shiftParticles, monomers unwrapped
      R wx = x.x, wy = x.y, wz = x.z, dvx = R(0);
      if (mono_bin == MONOBIN_WRAPPED) {
        img = static_cast<int>(r_round(wy / g.L[1]));
        le_wrap(g, wx, wy, wz, dvx);
      }
      const uint32_t c = cell_of(g, wx, wy, wz, strict != 0);
      if (c >= static_cast<uint32_t>(ri.n_cell)) {
        raise_error(err, ERR_MONO_CELL, static_cast<uint32_t>(r),
                    static_cast<uint32_t>(b - ri.mono_base + i));
      } else {
        key = static_cast<uint32_t>(ri.cell_base) + c;
      }
      // undo the shift right away: nothing reads monomer positions in between
      x.x += -s0; x.y += -s1; x.z += -s2;
      st4(mpos, b + i, x);
    }
    const uint32_t rank = warp_rank(count, key);
    if (i < n) {
      mkey[b + i] = make_uint2(key, rank);
      mimg[b + i] = img;
    }
  }
  if (frames != nullptr && threadIdx.x == 0 && blockIdx.y == 0) {
    FrameF f;
    for (int d = 0; d < 3; ++d) {
      f.L[d] = static_cast<float>(ri.L[d]);
      f.half[d] = 0.5f * static_cast<float>(ri.L[d]);
      f.Li[d] = ri.L[d];
      f.shift[d] = static_cast<float>(dn.shift[d]);
      f.com[d] = static_cast<float>(dn.com[d]);
      f.comv[d] = static_cast<float>(dn.comv[d]);
    }
    f.shear = static_cast<float>(ri.shear);
    f.shearLy = static_cast<float>(ri.shear * ri.L[1]);
    f.delrx = static_cast<float>(dn.delrx);
    f.h = static_cast<float>(dn.h);
    f.kT = static_cast<float>(ri.kT);
    f.solvent_mass = static_cast<float>(ri.solvent_mass);
    f.rot_c = static_cast<float>(rot_c);
    f.rot_s = static_cast<float>(rot_s);
    f.recentre = out;
    f.shear_on = ri.shear != 0.0;
    f.pad[0] = f.pad[1] = 0;
    frames[r] = f;
  }
}

// A cell key carried in a record's fourth word, as a bit pattern.
template <typename R>
__device__ __forceinline__ R key_word(uint32_t k);
template <>
__device__ __forceinline__ double key_word<double>(uint32_t k) {
  return __longlong_as_double(static_cast<long long>(k));
}
template <>
__device__ __forceinline__ float key_word<float>(uint32_t k) { return __uint_as_float(k); }
__device__ __forceinline__ uint32_t word_key(double w) {
  return static_cast<uint32_t>(__double_as_longlong(w));
}
__device__ __forceinline__ uint32_t word_key(float w) { return __float_as_uint(w); }

// Stream, shift, wrap and bin every solvent slot of a slot tile. Each thread
// loads U records (U independent 32-byte loads in flight), computes their
// keys, then takes ranks with warp-aggregated atomics whose U round trips
// overlap (all atomics are issued before any result is consumed).
// With frame, it also stores each binned particle's collision-frame record
// for the collide that follows (FP64 contexts: the collide then reads it
// instead of repeating the streaming, shift, wraps and cell index on the
// narrow FP64 pipe; the arithmetic is the same).
template <typename R, int NT>
__global__ void __launch_bounds__(NT) k_fluid_bin(const Tile* tiles, const RepInfo* reps,
                                                  const RepDyn* dyn, const R* __restrict__ st,
                                                  uint2* __restrict__ keys, uint32_t* count,
                                                  ErrorState* err, int strict, R* frame) {
  // FP64: two records in flight per thread, so that two blocks fit per SM
  // (the FP64 work is latency-bound on the narrow pipe; more warps hide it)
  constexpr int U = std::is_same<R, double>::value ? 2 : 4;
  const Tile t = tiles[blockIdx.x];
  const RepInfo& ri = reps[t.rep];
  const RepDyn dn = dyn[t.rep];
  const Geo<R> g = make_geo<R>(ri, dn, 0);
  const uint32_t cbase = static_cast<uint32_t>(ri.cell_base);
  const uint32_t ncell = static_cast<uint32_t>(ri.n_cell);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  for (int base = t.begin; base < t.end; base += NT * U) {
    R4<R> x[U], v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = base + u * NT + threadIdx.x;
      if (i < t.end) {
        x[u] = ld_pos(st, i);
        v[u] = ld_vel(st, i);
      }
    }
    uint32_t key[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = base + u * NT + threadIdx.x;
      key[u] = KEY_NONE;
      if (i < t.end && slot_id(x[u].w) != SLOT_EMPTY) {
        fluid_to_collision_frame(g, x[u], v[u]);
        const uint32_t c = cell_of(g, x[u].x, x[u].y, x[u].z, strict != 0);
        if (c >= ncell) {
          raise_error(err, ERR_FLUID_CELL, static_cast<uint32_t>(t.rep), static_cast<uint32_t>(i));
        } else {
          key[u] = cbase + c;
          // the collision-frame record for the collide, the key in the
          // velocity's fourth word (a bit pattern)
          if (frame) st_rec(frame, i, x[u], R4<R>{v[u].x, v[u].y, v[u].z, key_word<R>(key[u])});
        }
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
      if (i < t.end) keys[i] = make_uint2(key[u], b0 + __popc(peers[u] & below));
    }
  }
}

// perm[off[key] + rank] = source for every binned solvent slot and monomer.
__global__ void k_build_perm(const uint2* __restrict__ keys, int n_slots,
                             const uint2* __restrict__ mkey, int n_mono,
                             const uint32_t* __restrict__ off, uint32_t* __restrict__ perm,
                             ErrorState* err);

// --------------------------------------------------------- collide

template <typename R>
struct AccT;
template <>
struct AccT<double> {
  typedef double type;
};
template <>
struct AccT<float> {
  typedef long long type;  // 2^32 fixed point: exact, order-independent sums
};


// One term of a cell sum; the FP32 form also keeps the largest |v| converted
// in `big` (fixed-point range check, precision.cuh).
template <typename R>
__device__ __forceinline__ typename AccT<R>::type to_acc(R v, float& big);
template <>
__device__ __forceinline__ double to_acc<double>(double v, float&) { return v; }
template <>
__device__ __forceinline__ long long to_acc<float>(float v, float& big) {
  big = fmaxf(big, fabsf(v));
  return f2fix32(v);
}

__device__ __forceinline__ float acc_to_float(long long a) { return fix32_to_f(a); }

// A particle of a collide tile in the collision frame.
template <typename R>
struct Particle {
  R4<R> x;   // shifted, wrapped position (solvent); .w: particle id
  R4<R> v;   // velocity in the primary box frame
  R m;
  int lc;    // local cell in the tile, -1 for an idle lane
  uint32_t src;
};

__device__ __forceinline__ float pack_src(float, uint32_t s) { return __uint_as_float(s); }
__device__ __forceinline__ double pack_src(double, uint32_t s) { return make_slot_id<double>(s); }
__device__ __forceinline__ uint32_t unpack_src(float w) { return __float_as_uint(w); }
__device__ __forceinline__ uint32_t unpack_src(double w) { return slot_id(w); }

template <typename R>
struct CollideCtx {
  const uint32_t* __restrict__ perm;
  const R* __restrict__ st;
  // collision-frame records the binning wrote (solvent slots: streamed,
  // shifted, wrapped position with the id; velocity with the cell key), or
  // null: recomputed from st
  const R* __restrict__ fr;
  const R* mpos;
  R* mvel;
  const uint2* mkey;
  const int* mimg;
  Geo<R> g;
  RepDyn dn;
  R solvent_mass;
  uint32_t cbase;
  uint32_t c0;
  int nc;
  bool strict;
  bool amc;  // angular-momentum-conserving collision: monomers need positions
  ErrorState* err;
};

// Reconstructs sorted position p of the tile from global memory (the gather
// stage and the overflow path share it).
template <typename R>
__device__ __forceinline__ void finish_particle(Particle<R>& P, uint32_t p, const CollideCtx<R>& C) {
  if (P.src & MONO_BIT) {
    const uint32_t m = P.src & ~MONO_BIT;
    if (C.g.wrap_mono == MONOBIN_WRAPPED)
      P.v.x = r_sub(P.v.x, r_mul(r_mul(static_cast<R>(C.mimg[m]), C.g.shear), C.g.L[1]));
    if (C.amc) {
      // the monomer where k_mono_prep binned it: shifted, at its image when
      // monomers are binned wrapped
      const R4<R> x = ld4_rw(C.mpos, m);
      P.x.x = x.x + C.g.shift[0];
      P.x.y = x.y + C.g.shift[1];
      P.x.z = x.z + C.g.shift[2];
      if (C.g.wrap_mono == MONOBIN_WRAPPED) {
        R dvx = R(0);
        le_wrap(C.g, P.x.x, P.x.y, P.x.z, dvx);
      }
    }
    P.lc = static_cast<int>(C.mkey[m].x - C.c0);
  } else if (C.fr) {
    P.m = C.solvent_mass;
    P.lc = static_cast<int>(word_key(P.v.w) - C.c0);
  } else {
    fluid_to_collision_frame(C.g, P.x, P.v);
    P.m = C.solvent_mass;
    const uint32_t c = cell_of(C.g, P.x.x, P.x.y, P.x.z, C.strict);
    P.lc = static_cast<int>(C.cbase + c - C.c0);
  }
  if (P.lc < 0 || P.lc >= C.nc) {  // cannot happen when binning and recompute agree
    raise_error(C.err, ERR_KEY_MISMATCH, p, P.src);
    P.lc = -1;
  }
}

template <typename R>
__device__ __forceinline__ void fetch_raw(Particle<R>& P, uint32_t src, const CollideCtx<R>& C) {
  P.src = src;
  if (src & MONO_BIT) {
    const uint32_t m = src & ~MONO_BIT;
    P.v = ld4_rw(C.mvel, m);
    P.m = ld4_rw(C.mpos, m).w;
  } else {
    const R* s = C.fr ? C.fr : C.st;
    P.x = ld_pos(s, src);
    P.v = ld_vel(s, src);
  }
}

template <typename R>
__device__ __forceinline__ void load_particle(Particle<R>& P, uint32_t p, uint32_t p1,
                                              const CollideCtx<R>& C) {
  P.lc = -1;
  if (p >= p1) return;
  fetch_raw(P, C.perm[p], C);
  finish_particle(P, p, C);
}

// Sign and finiteness tests of a per-particle value without FP64 compares:
// on GB300 DSETP issues on the narrow FP64 pipe, the integer tests do not.
// not_negative(x) is x >= 0 for every double: +0 up to +inf are the bit
// patterns 0 .. 0x7FF0000000000000, and -0.0 compares equal to 0; NaNs and
// negative numbers are false.
__device__ __forceinline__ bool not_negative(float x) { return x >= 0.0f; }
__device__ __forceinline__ bool not_negative(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  return b <= 0x7FF0000000000000ull || b == 0x8000000000000000ull;
}
__device__ __forceinline__ bool finite_bits(float x) { return isfinite(x); }
__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7FF) != 0x7FF;
}

// Thermostat + rotation of one particle, then the unshift/wrap and store.
template <typename R>
__device__ __forceinline__ void apply_collision(Particle<R>& P, uint32_t p, const R* s_cmv,
                                                const R* s_rot, const R* s_scale,
                                                const R* s_ang, const R* s_cmp,
                                                const CollideCtx<R>& C, R* st_out,
                                                ErrorState* err) {
  if (P.lc < 0) return;
  const R* cm = s_cmv + 3 * P.lc;
  const R* M = s_rot + 9 * P.lc;
  const R sc = s_scale[P.lc];
  R vx = P.v.x, vy = P.v.y, vz = P.v.z;
  R d0, d1, d2;
  if (std::is_same<R, double>::value) {
    // MPC.cpp:291 then MPC.cpp:267, in the reference's operation order
    if (not_negative(sc)) {
      vx = sc * vx + (R(1) - sc) * cm[0];
      vy = sc * vy + (R(1) - sc) * cm[1];
      vz = sc * vz + (R(1) - sc) * cm[2];
    }
    d0 = vx - cm[0];
    d1 = vy - cm[1];
    d2 = vz - cm[2];
  } else {
    const R f = sc >= R(0) ? sc : R(1);
    d0 = (vx - cm[0]) * f;
    d1 = (vy - cm[1]) * f;
    d2 = (vz - cm[2]) * f;
  }
  vx = cm[0] + ((M[0] * d0 + M[1] * d1) + M[2] * d2);
  vy = cm[1] + ((M[3] * d0 + M[4] * d1) + M[5] * d2);
  vz = cm[2] + ((M[6] * d0 + M[7] * d1) + M[8] * d2);
  if (C.amc) {  // + Angular x (r - CMP) (MPC.cpp:268); zero outside AMC cells
    const R* w = s_ang + 3 * P.lc;
    const R* c = s_cmp + 3 * P.lc;
    const R q0 = P.x.x - c[0], q1 = P.x.y - c[1], q2 = P.x.z - c[2];
    vx += w[1] * q2 - w[2] * q1;
    vy += w[2] * q0 - w[0] * q2;
    vz += w[0] * q1 - w[1] * q0;
  }
  if (!(finite_bits(vx) && finite_bits(vy) && finite_bits(vz)))
    raise_error(err, ERR_NONFINITE, p, P.src);
  if (P.src & MONO_BIT) {
    const uint32_t m = P.src & ~MONO_BIT;
    if (C.g.wrap_mono == MONOBIN_WRAPPED)
      vx = r_add(vx, r_mul(r_mul(static_cast<R>(C.mimg[m]), C.g.shear), C.g.L[1]));
    R4<R> v = ld4_rw(C.mvel, m);
    v.x = vx;
    v.y = vy;
    v.z = vz;
    st4(C.mvel, m, v);
    st_rec(st_out, p, R4<R>{R(0), R(0), R(0), make_slot_id<R>(SLOT_EMPTY)},
           R4<R>{R(0), R(0), R(0), R(0)});
  } else {
    R4<R> x = P.x;
    x.x = r_add(x.x, -C.g.shift[0]);
    x.y = r_add(x.y, -C.g.shift[1]);
    x.z = r_add(x.z, -C.g.shift[2]);
    le_wrap(C.g, x.x, x.y, x.z, vx);  // x.w: the particle id, carried through
    st_rec(st_out, p, x, R4<R>{vx, vy, vz, R(0)});
  }
}

// Dynamic shared memory of k_collide: CAP staged particles (position and
// velocity records, 16-bit local cell).
template <typename R>
constexpr size_t collide_dyn_smem(int cap) {
  return static_cast<size_t>(cap) * (2 * sizeof(R4<R>) + sizeof(short));
}

// Staged particle j of the tile (shared memory), or, past the staging
// capacity, reconstructed from global memory.
template <typename R, int CAP>
__device__ __forceinline__ void tile_particle(Particle<R>& P, int j, int nloc, uint32_t p0,
                                              uint32_t p1, const R4<R>* s_x, const R4<R>* s_v,
                                              const short* s_lc, const CollideCtx<R>& C) {
  if (j < nloc) {
    P.x = s_x[j];
    P.v = s_v[j];
    P.m = P.v.w;
    P.lc = s_lc[j];
    P.src = unpack_src(P.x.w);  // solvent id (no MONO_BIT) or MONO_BIT | monomer
  } else {
    load_particle(P, p0 + j, p1, C);
  }
}


template <typename R>
__device__ __forceinline__ R acc_to_r(typename AccT<R>::type a);
template <>
__device__ __forceinline__ double acc_to_r<double>(double a) { return a; }
template <>
__device__ __forceinline__ float acc_to_r<float>(long long a) { return fix32_to_f(a); }

__device__ __forceinline__ long long shfl_pair(long long v) {
  return __shfl_xor_sync(0xFFFFFFFFu, v, 1);
}
__device__ __forceinline__ double shfl_pair(double v) {
  return __shfl_xor_sync(0xFFFFFFFFu, v, 1);
}

// x = A^-1 b for a symmetric positive-definite 3x3 A: the Cholesky factor
// A = L L^T column by column, forward then back substitution (the LLT solve
// MPC::calculateAngular calls, MPC.cpp:373).
template <typename R>
__device__ __forceinline__ void llt_solve3(const R A[3][3], const R b[3], R x[3]) {
  R l[3][3] = {{R(0), R(0), R(0)}, {R(0), R(0), R(0)}, {R(0), R(0), R(0)}}, y[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    R s = A[j][j];
    for (int k = 0; k < j; ++k) s -= l[j][k] * l[j][k];
    l[j][j] = r_sqrt(s);
    for (int i = j + 1; i < 3; ++i) {
      R t = A[i][j];
      for (int k = 0; k < j; ++k) t -= l[i][k] * l[j][k];
      l[i][j] = t / l[j][j];
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R s = b[i];
    for (int k = 0; k < i; ++k) s -= l[i][k] * y[k];
    y[i] = s / l[i][i];
  }
#pragma unroll
  for (int i = 2; i >= 0; --i) {
    R s = y[i];
    for (int k = i + 1; k < 3; ++k) s -= l[k][i] * x[k];
    x[i] = s / l[i][i];
  }
}

// Thermostat factor of one cell (MPC.cpp:284-291): sqrt(Gamma(1.5 (n - 1),
// kT) / E) for cells of two or more particles, -1 (no thermostat) otherwise.
template <typename R>
__device__ __forceinline__ R cell_scale(uint32_t nn, R ekin, uint32_t cg, uint32_t cl, int rng,
                                        const double* inj_gamma, unsigned long long seed,
                                        unsigned long long step, R kT, ErrorState* err) {
  constexpr bool kFP64 = std::is_same<R, double>::value;
  if (nn < 2u) return R(-1);
  R gv;
  if (rng == RNG_INJECT) {
    gv = static_cast<R>(inj_gamma[cg]);
  } else {
    bool ok = true;
    const R shape = kFP64 ? static_cast<R>(1.5) * static_cast<R>(nn - 1u)
                          : static_cast<R>(1.5f * i2f_small(static_cast<int>(nn - 1u)));
    gv = philox_gamma<R>(seed, cl, step, shape, &ok) * kT;
    if (!ok) raise_error(err, ERR_GAMMA_ITERS, cg, nn);
  }
  return (ekin > R(0)) ? r_sqrt(gv / ekin) : R(1);
}

// Rotation matrix of one cell about the random axis (MPC.cpp:244-257).
template <typename R>
__device__ __forceinline__ void cell_rotation(uint32_t cg, uint32_t cl, int rng,
                                              const double* inj_uphi, const double* inj_utheta,
                                              unsigned long long seed, unsigned long long step,
                                              R rc, R rs, R (&M)[9]) {
  R uphi, uth;
  if (rng == RNG_INJECT) {
    uphi = static_cast<R>(inj_uphi[cg]);
    uth = static_cast<R>(inj_utheta[cg]);
  } else {
    const Uniform2<R> u = philox_uniforms<R>(seed, cl, step, 0u);
    uphi = u.a;
    uth = u.b;
  }
  const R two_pi = R(6.283185307179586476925286766559);
  const R phi = two_pi * uphi;
  const R theta = R(2) * (uth - R(0.5));
  const R stt = r_sqrt(R(1) - theta * theta);
  R sphi, cphi;
  r_sincos(phi, &sphi, &cphi);
  const R a0 = stt * cphi, a1 = stt * sphi, a2 = theta;
  M[0] = a0 * a0 + (R(1) - a0 * a0) * rc;
  M[1] = a0 * a1 * (R(1) - rc) - a2 * rs;
  M[2] = a0 * a2 * (R(1) - rc) + a1 * rs;
  M[3] = a0 * a1 * (R(1) - rc) + a2 * rs;
  M[4] = a1 * a1 + (R(1) - a1 * a1) * rc;
  M[5] = a1 * a2 * (R(1) - rc) - a0 * rs;
  M[6] = a0 * a2 * (R(1) - rc) - a1 * rs;
  M[7] = a1 * a2 * (R(1) - rc) + a0 * rs;
  M[8] = a2 * a2 + (R(1) - a2 * a2) * rc;
}

// One CTA per tile of <= CT cells of one replica.
//  stage  : gather the tile's particles (perm -> 32-byte records, GU loads in
//           flight per thread), recompute their collision-frame state, keep
//           them in shared memory;
//  cells  : one thread per cell walks its particles twice -- momentum and
//           mass (MPC::calculateCMV, MPC.cpp:314-322), then kinetic energy
//           about the cell velocity (MPC.cpp:277-280) -- with int64 fixed-point
//           sums on the fast path (exact, independent of particle order) and
//           the reference's sequential FP64 sums on the parity path; then
//           draws the MBS factor (MPC.cpp:287-289) and the rotation
//           (MPC.cpp:244-257);
//  amc    : (angular-momentum-conserving collision, cells of more than two
//           particles) the cell's centre of mass, the angular momentum the
//           rotation removed and the inertia tensor, summed by the same two
//           lanes about the cell's corner (FP32: fixed point), and the
//           angular velocity that puts it back (MPC.cpp:260-269, 324-374);
//  apply  : rotate/scale (+ angular term), undo the shift, write the tile
//           back in cell order.
// A tile holding more than CAP particles reads the excess straight from
// global memory (correct, slower).
template <typename R, int NT, int CT, int CAP>
__global__ void __launch_bounds__(NT) k_collide(
    const Tile* tiles, const RepInfo* reps, const RepDyn* dyn, const uint32_t* __restrict__ off,
    const uint32_t* __restrict__ perm, const R* __restrict__ st_in, R* __restrict__ st_out,
    const R* mpos, R* mvel, const uint2* mkey, const int* mimg, const double* inj_gamma,
    const double* inj_uphi, const double* inj_utheta, int rng, double rot_c, double rot_s,
    int strict, int mono_bin, int amc, ErrorState* err, const R* frame) {
  constexpr int GU = 4;
  constexpr bool kFP64 = std::is_same<R, double>::value;
  typedef typename AccT<R>::type Acc;
  __shared__ R s_cmv[CT * 3];
  __shared__ R s_rot[CT * 9];
  __shared__ R s_scale[CT];
  __shared__ R s_ang[CT * 3];
  __shared__ R s_cmp[CT * 3];
  __shared__ uint32_t s_off[CT + 1];
  extern __shared__ __align__(16) unsigned char s_dyn[];
  R4<R>* s_x = reinterpret_cast<R4<R>*>(s_dyn);
  R4<R>* s_v = s_x + CAP;
  short* s_lc = reinterpret_cast<short*>(s_v + CAP);

  const Tile t = tiles[blockIdx.x];
  const RepInfo& ri = reps[t.rep];
  CollideCtx<R> C;
  C.perm = perm;
  C.st = st_in;
  C.fr = frame;
  C.mpos = mpos;
  C.mvel = mvel;
  C.mkey = mkey;
  C.mimg = mimg;
  C.dn = dyn[t.rep];
  C.g = make_geo<R>(ri, C.dn, mono_bin);
  C.solvent_mass = static_cast<R>(ri.solvent_mass);
  C.cbase = static_cast<uint32_t>(ri.cell_base);
  C.c0 = static_cast<uint32_t>(t.begin);
  C.strict = strict != 0;
  C.amc = amc != 0;
  const int nc = t.end - t.begin;
  C.nc = nc;
  C.err = err;
  const R rc = static_cast<R>(rot_c), rs = static_cast<R>(rot_s);
  const R kT = static_cast<R>(ri.kT);

  for (int i = threadIdx.x; i <= nc; i += NT) s_off[i] = off[t.begin + i];
  __syncthreads();
  const uint32_t p0 = s_off[0], p1 = s_off[nc];
  const int n = static_cast<int>(p1 - p0);
  const int nloc = n < CAP ? n : CAP;

  // stage
  for (int base = 0; base < nloc; base += NT * GU) {
    uint32_t src[GU];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int j = base + u * NT + threadIdx.x;
      src[u] = j < nloc ? perm[p0 + j] : 0u;
    }
    Particle<R> P[GU];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int j = base + u * NT + threadIdx.x;
      if (j < nloc) fetch_raw(P[u], src[u], C);
    }
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      const int j = base + u * NT + threadIdx.x;
      if (j < nloc) {
        finish_particle(P[u], p0 + j, C);
        R4<R> x = P[u].x;  // solvent: .w keeps the particle id
        if (P[u].src & MONO_BIT) x.w = pack_src(R(0), P[u].src);
        R4<R> v = P[u].v;
        v.w = P[u].m;
        s_x[j] = x;
        s_v[j] = v;
        s_lc[j] = static_cast<short>(P[u].lc);
      }
    }
  }
  __syncthreads();

  // cells: two lanes per cell (NT == 2 CT) each walk half of its particles;
  // partial sums meet through one shuffle. Then lane 0 of the pair draws the
  // gamma variate while lane 1 builds the rotation.
  static_assert(NT == 2 * CT, "two threads per cell");
  {
    const int lc = threadIdx.x >> 1;
    const int half = threadIdx.x & 1;
    const bool live = lc < nc;
    const int j0 = live ? static_cast<int>(s_off[lc] - p0) : 0;
    const int j1 = live ? static_cast<int>(s_off[lc + 1] - p0) : 0;
    R cm[3];
    R ekin = R(0);
    float fix_big = 0.0f;  // FP32: largest fixed-point term (range check)
    if (kFP64) {
      R px = R(0), py = R(0), pz = R(0), mt = R(0);
      for (int j = j0 + half; j < j1; j += 2) {
        Particle<R> P;
        tile_particle<R, CAP>(P, j, nloc, p0, p1, s_x, s_v, s_lc, C);
        if (P.lc < 0) continue;
        px += P.v.x * P.m;
        py += P.v.y * P.m;
        pz += P.v.z * P.m;
        mt += P.m;
      }
      px += __shfl_xor_sync(0xFFFFFFFFu, px, 1);
      py += __shfl_xor_sync(0xFFFFFFFFu, py, 1);
      pz += __shfl_xor_sync(0xFFFFFFFFu, pz, 1);
      mt += __shfl_xor_sync(0xFFFFFFFFu, mt, 1);
      cm[0] = px; cm[1] = py; cm[2] = pz;
      if (mt > R(0)) {
        cm[0] /= mt; cm[1] /= mt; cm[2] /= mt;
      }
      for (int j = j0 + half; j < j1; j += 2) {
        Particle<R> P;
        tile_particle<R, CAP>(P, j, nloc, p0, p1, s_x, s_v, s_lc, C);
        if (P.lc < 0) continue;
        const R d0 = P.v.x - cm[0], d1 = P.v.y - cm[1], d2 = P.v.z - cm[2];
        ekin += P.m * ((d0 * d0 + d1 * d1) + d2 * d2);
      }
      ekin += __shfl_xor_sync(0xFFFFFFFFu, ekin, 1);
      ekin *= R(0.5);
    } else {
      // int64 2^32 fixed point: exact and independent of particle order.
      // Mass: solvent count times the solvent mass plus the monomers' masses.
      long long px = 0, py = 0, pz = 0, e = 0;
      int nsol = 0;
      float mmono = 0.0f;
      for (int j = j0 + half; j < j1; j += 2) {
        Particle<R> P;
        tile_particle<R, CAP>(P, j, nloc, p0, p1, s_x, s_v, s_lc, C);
        if (P.lc < 0) continue;
        px += to_acc<R>(P.v.x * P.m, fix_big);
        py += to_acc<R>(P.v.y * P.m, fix_big);
        pz += to_acc<R>(P.v.z * P.m, fix_big);
        if (P.src & MONO_BIT) {
          mmono += static_cast<float>(P.m);
        } else {
          ++nsol;
        }
      }
      px += __shfl_xor_sync(0xFFFFFFFFu, px, 1);
      py += __shfl_xor_sync(0xFFFFFFFFu, py, 1);
      pz += __shfl_xor_sync(0xFFFFFFFFu, pz, 1);
      nsol += __shfl_xor_sync(0xFFFFFFFFu, nsol, 1);
      mmono += __shfl_xor_sync(0xFFFFFFFFu, mmono, 1);
      const float mt = fmaf(i2f_small(nsol), static_cast<float>(C.solvent_mass), mmono);
      const float inv = mt > 0.f ? 1.0f / mt : 0.0f;
      cm[0] = acc_to_float(px) * inv;
      cm[1] = acc_to_float(py) * inv;
      cm[2] = acc_to_float(pz) * inv;
      for (int j = j0 + half; j < j1; j += 2) {
        Particle<R> P;
        tile_particle<R, CAP>(P, j, nloc, p0, p1, s_x, s_v, s_lc, C);
        if (P.lc < 0) continue;
        const R d0 = P.v.x - cm[0], d1 = P.v.y - cm[1], d2 = P.v.z - cm[2];
        e += to_acc<R>(P.m * ((d0 * d0 + d1 * d1) + d2 * d2), fix_big);
      }
      e += __shfl_xor_sync(0xFFFFFFFFu, e, 1);
      ekin = acc_to_float(e) * 0.5f;
    }
    const uint32_t cg = C.c0 + lc;
    const uint32_t cl = cg - C.cbase;
    const uint32_t nn = static_cast<uint32_t>(j1 - j0);
    R scale = R(-1);
    R M[9];
    if (kFP64 && !amc) {
      // FP64: the draws of each cell by one thread, in full warps. On the two
      // lanes of a pair the gamma variate and the rotation take divergent
      // paths, each at half the warp, and the narrow FP64 pipe issues every
      // warp instruction for the whole warp.
      if (half == 0 && live) {
        s_cmv[3 * lc] = cm[0];
        s_cmv[3 * lc + 1] = cm[1];
        s_cmv[3 * lc + 2] = cm[2];
        s_scale[lc] = ekin;
      }
      __syncthreads();
      for (int c = threadIdx.x; c < nc; c += NT) {
        const uint32_t cgc = C.c0 + c;
        const uint32_t nnc = s_off[c + 1] - s_off[c];
        R Mc[9];
        const R sc = cell_scale<R>(nnc, s_scale[c], cgc, cgc - C.cbase, rng, inj_gamma, ri.seed,
                                   C.dn.step, kT, err);
        cell_rotation<R>(cgc, cgc - C.cbase, rng, inj_uphi, inj_utheta, ri.seed, C.dn.step, rc,
                         rs, Mc);
#pragma unroll
        for (int q = 0; q < 9; ++q) s_rot[9 * c + q] = Mc[q];
        s_scale[c] = sc;
      }
      __syncthreads();
      goto apply;
    }
    if (half == 0) {
      if (live) scale = cell_scale<R>(nn, ekin, cg, cl, rng, inj_gamma, ri.seed, C.dn.step, kT, err);
    } else if (live) {
      cell_rotation<R>(cg, cl, rng, inj_uphi, inj_utheta, ri.seed, C.dn.step, rc, rs, M);
    }
    {  // both lanes get lane 0's factor
      const R other = __shfl_xor_sync(0xFFFFFFFFu, scale, 1);
      if (half == 1) scale = other;
    }
    R ang[3] = {R(0), R(0), R(0)}, cmp[3] = {R(0), R(0), R(0)};
    if (amc) {  // uniform over the CTA
#pragma unroll
      for (int q = 0; q < 9; ++q) {  // lane 0 takes lane 1's rotation
        const R o = __shfl_xor_sync(0xFFFFFFFFu, M[q], 1);
        if (half == 0) M[q] = o;
      }
      const bool cell_amc = live && nn > 2u;
      // the cell's corner in the collision frame (cell index = floor(x + L/2))
      const int Lx = ri.L[0], Ly = ri.L[1];
      const int ix = static_cast<int>(cl % static_cast<uint32_t>(Lx));
      const int iy = static_cast<int>((cl / static_cast<uint32_t>(Lx)) % static_cast<uint32_t>(Ly));
      const int iz = static_cast<int>(cl / static_cast<uint32_t>(Lx * Ly));
      const R k0 = static_cast<R>(ix) - C.g.half[0], k1 = static_cast<R>(iy) - C.g.half[1],
              k2 = static_cast<R>(iz) - C.g.half[2];
      Acc s0 = 0, s1 = 0, s2 = 0, sm = 0;
      for (int j = j0 + half; cell_amc && j < j1; j += 2) {
        Particle<R> P;
        tile_particle<R, CAP>(P, j, nloc, p0, p1, s_x, s_v, s_lc, C);
        if (P.lc < 0) continue;
        s0 += to_acc<R>((P.x.x - k0) * P.m, fix_big);
        s1 += to_acc<R>((P.x.y - k1) * P.m, fix_big);
        s2 += to_acc<R>((P.x.z - k2) * P.m, fix_big);
        sm += to_acc<R>(P.m, fix_big);
      }
      s0 += shfl_pair(s0);
      s1 += shfl_pair(s1);
      s2 += shfl_pair(s2);
      sm += shfl_pair(sm);
      const R mt = acc_to_r<R>(sm);
      const R c0 = mt > R(0) ? acc_to_r<R>(s0) / mt : R(0);
      const R c1 = mt > R(0) ? acc_to_r<R>(s1) / mt : R(0);
      const R c2 = mt > R(0) ? acc_to_r<R>(s2) / mt : R(0);
      // angular momentum the rotation removes, and the inertia tensor
      Acc a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      const R f = scale >= R(0) ? scale : R(1);
      for (int j = j0 + half; cell_amc && j < j1; j += 2) {
        Particle<R> P;
        tile_particle<R, CAP>(P, j, nloc, p0, p1, s_x, s_v, s_lc, C);
        if (P.lc < 0) continue;
        const R q0 = (P.x.x - k0) - c0, q1 = (P.x.y - k1) - c1, q2 = (P.x.z - k2) - c2;
        R u0, u1, u2;
        if (kFP64 && scale >= R(0)) {  // the thermostatted velocity (MPC.cpp:291)
          u0 = (scale * P.v.x + (R(1) - scale) * cm[0]) - cm[0];
          u1 = (scale * P.v.y + (R(1) - scale) * cm[1]) - cm[1];
          u2 = (scale * P.v.z + (R(1) - scale) * cm[2]) - cm[2];
        } else {
          u0 = (P.v.x - cm[0]) * f;
          u1 = (P.v.y - cm[1]) * f;
          u2 = (P.v.z - cm[2]) * f;
        }
        const R w0 = u0 - ((M[0] * u0 + M[1] * u1) + M[2] * u2);
        const R w1 = u1 - ((M[3] * u0 + M[4] * u1) + M[5] * u2);
        const R w2 = u2 - ((M[6] * u0 + M[7] * u1) + M[8] * u2);
        a[0] += to_acc<R>(P.m * (q1 * w2 - q2 * w1), fix_big);
        a[1] += to_acc<R>(P.m * (q2 * w0 - q0 * w2), fix_big);
        a[2] += to_acc<R>(P.m * (q0 * w1 - q1 * w0), fix_big);
        a[3] += to_acc<R>(P.m * (q1 * q1 + q2 * q2), fix_big);
        a[4] += to_acc<R>(P.m * (q0 * q0 + q2 * q2), fix_big);
        a[5] += to_acc<R>(P.m * (q1 * q1 + q0 * q0), fix_big);
        a[6] += to_acc<R>(P.m * q0 * q1, fix_big);
        a[7] += to_acc<R>(P.m * q0 * q2, fix_big);
        a[8] += to_acc<R>(P.m * q1 * q2, fix_big);
      }
#pragma unroll
      for (int q = 0; q < 9; ++q) a[q] += shfl_pair(a[q]);
      if (cell_amc) {
        const R I[3][3] = {{acc_to_r<R>(a[3]), -acc_to_r<R>(a[6]), -acc_to_r<R>(a[7])},
                           {-acc_to_r<R>(a[6]), acc_to_r<R>(a[4]), -acc_to_r<R>(a[8])},
                           {-acc_to_r<R>(a[7]), -acc_to_r<R>(a[8]), acc_to_r<R>(a[5])}};
        const R cv[3] = {acc_to_r<R>(a[0]), acc_to_r<R>(a[1]), acc_to_r<R>(a[2])};
        llt_solve3<R>(I, cv, ang);
        cmp[0] = k0 + c0;
        cmp[1] = k1 + c1;
        cmp[2] = k2 + c2;
      }
    }
    if (!kFP64 && fix_big >= FIX32_LIMIT)
      raise_error(err, ERR_FIXPOINT, C.c0 + lc, __float_as_uint(fix_big));
    if (half == 1 && live) {
      s_ang[3 * lc] = ang[0];
      s_ang[3 * lc + 1] = ang[1];
      s_ang[3 * lc + 2] = ang[2];
      s_cmp[3 * lc] = cmp[0];
      s_cmp[3 * lc + 1] = cmp[1];
      s_cmp[3 * lc + 2] = cmp[2];
    }
    if (half == 1 && live) {
      if (!kFP64 && scale >= R(0)) {
#pragma unroll
        for (int q = 0; q < 9; ++q) M[q] *= scale;  // fast path: s R in one matrix
      }
#pragma unroll
      for (int q = 0; q < 9; ++q) s_rot[9 * lc + q] = M[q];
      s_cmv[3 * lc] = cm[0];
      s_cmv[3 * lc + 1] = cm[1];
      s_cmv[3 * lc + 2] = cm[2];
      s_scale[lc] = kFP64 ? scale : R(-1);
    }
  }
  __syncthreads();

apply:
  for (int j = threadIdx.x; j < nloc; j += NT) {
    Particle<R> P;
    tile_particle<R, CAP>(P, j, nloc, p0, p1, s_x, s_v, s_lc, C);
    apply_collision(P, p0 + j, s_cmv, s_rot, s_scale, s_ang, s_cmp, C, st_out, err);
  }
  for (int base = CAP; base < n; base += NT) {
    Particle<R> P;
    load_particle(P, p0 + base + threadIdx.x, p1, C);
    apply_collision(P, p0 + base + threadIdx.x, s_cmv, s_rot, s_scale, s_ang, s_cmp, C, st_out,
                    err);
  }
}

// Solvent temperature on the last collision's cells (MPC.cpp:384-418):
// CMV over every particle of a cell, kinetic energy over its solvent only.
// One thread per cell; per-tile FP64 partial sums.
template <typename R, int NT>
__global__ void __launch_bounds__(NT) k_temperature(
    const Tile* tiles, const RepInfo* reps, const uint32_t* __restrict__ off,
    const uint32_t* __restrict__ perm, const R* __restrict__ st_cur, const R* mpos,
    const R* mvel, const int* mimg, int mono_bin, TempPartial* partial) {
  __shared__ double s_e[NT];
  __shared__ unsigned s_f[NT];
  const Tile t = tiles[blockIdx.x];
  const RepInfo& ri = reps[t.rep];
  const double shearLy = ri.shear * static_cast<double>(ri.L[1]);
  double e_sum = 0.0;
  unsigned filled = 0;
  for (int c = t.begin + threadIdx.x; c < t.end; c += NT) {
    const uint32_t a = off[c], b = off[c + 1];
    double px = 0, py = 0, pz = 0, mt = 0;
    unsigned nf = 0;
    for (uint32_t p = a; p < b; ++p) {
      const uint32_t src = perm[p];
      double vx, vy, vz, m;
      if (src & MONO_BIT) {
        const uint32_t mi = src & ~MONO_BIT;
        const R4<R> v = ld4_rw(mvel, mi);
        m = static_cast<double>(ld4_rw(mpos, mi).w);
        vx = v.x; vy = v.y; vz = v.z;
        if (mono_bin == MONOBIN_WRAPPED) vx -= static_cast<double>(mimg[mi]) * shearLy;
      } else {
        const R4<R> v = ld_vel(st_cur, p);
        m = ri.solvent_mass;
        vx = v.x; vy = v.y; vz = v.z;
        ++nf;
      }
      px += vx * m; py += vy * m; pz += vz * m; mt += m;
    }
    if (mt > 0) { px /= mt; py /= mt; pz /= mt; }
    double ek = 0.0;
    for (uint32_t p = a; p < b; ++p) {
      if (perm[p] & MONO_BIT) continue;
      const R4<R> v = ld_vel(st_cur, p);
      const double d0 = v.x - px, d1 = v.y - py, d2 = v.z - pz;
      ek += ri.solvent_mass * ((d0 * d0 + d1 * d1) + d2 * d2);
    }
    e_sum += ek * 0.5;
    filled += nf > 0 ? 1u : 0u;
  }
  s_e[threadIdx.x] = e_sum;
  s_f[threadIdx.x] = filled;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s_e[threadIdx.x] += s_e[threadIdx.x + s];
      s_f[threadIdx.x] += s_f[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[blockIdx.x].ekin = s_e[0];
    partial[blockIdx.x].filled = s_f[0];
  }
}

}  // namespace smpc
