// Monomer velocity-Verlet substeps (Thermostat_None::propagate,
// star-polymers/lib/Thermostats/Thermostat_None.cpp:21-38) with the
// displacement-triggered Verlet list (Box::check_VerletLists /
// update_VerletLists, star-polymers/lib/Box.cpp:105-194) and the FENE + pair
// forces (Box::calculate_forces_verlet, Box.cpp:243-286; potentials
// star-polymers/lib/Molecules/Potentials.h:14-120).
//
// One CTA per replica runs all n substeps of a call: positions live in
// shared memory (other threads read them for forces), each thread owns up to
// MPT monomers in registers (v, F, Verlet reference position). Forces are
// computed per bead over its own Verlet list and its own undirected bond
// list, so no atomics and no write conflicts; the reference's directed bond
// (F_src -= f d, F_dst += f d) is the same force seen from both ends.
//
// With KMAX > 1 (one bead per thread, MPT = 1) a replica with n beads gives
// each bead k = the largest power of two <= min(KMAX, NT / n) adjacent lanes:
// all k hold the bead's state, each walks every k-th entry of its Verlet
// list, and a butterfly over the k lanes sums the partial forces. Small
// replicas then use the whole CTA instead of n of its threads.
#pragma once
#include <cooperative_groups.h>
#include <stdint.h>

#include "mpc_kernels.cuh"
#include "smpc_device.cuh"

namespace smpc {

// r2 < c for a squared distance r2 (a sum of squares: +0 or more, or NaN)
// and a cut-off c > 0. In FP64 the comparison runs on the bit patterns,
// whose unsigned integer order is the numeric order for non-negative doubles
// (NaN patterns lie above every finite one, so a NaN r2 compares false as in
// FP64), and does not take the narrow FP64 pipe.
__device__ __forceinline__ bool r2_below(double r2, double c) {
  return static_cast<unsigned long long>(__double_as_longlong(r2)) <
         static_cast<unsigned long long>(__double_as_longlong(c));
}
__device__ __forceinline__ bool r2_below(float r2, float c) { return r2 < c; }

// Pair force magnitude f such that F_i -= f (x_j - x_i).
template <typename R>
__device__ __forceinline__ R pair_force(int pot, bool bb, R r2, R lambda) {
  if (pot == POT_REF4824) {
    // TypeAA_Force / TypeBB_Force (Potentials.h:57-120)
    if (r2_below(r2, R(1.0594631))) {
      const R rm2 = R(1) / r2;
      R rm24 = rm2 * rm2 * rm2;
      rm24 *= rm24;
      rm24 *= rm24;
      return R(192.0) * rm2 * rm24 * (rm24 - R(0.5));
    }
    if (bb && r2_below(r2, R(2.25))) {
      const R rm2 = R(1) / r2;
      R rm24 = rm2 * rm2 * rm2;
      rm24 *= rm24;
      rm24 *= rm24;
      return R(192.0) * lambda * rm2 * rm24 * (rm24 - R(0.5));
    }
    return R(0);
  }
  // 12-6 preset: WCA core for all pairs, lambda-scaled LJ attraction to 2.5 for BB
  const bool core = r2_below(r2, R(1.2599210498948732));
  if (core || (bb && r2_below(r2, R(6.25)))) {
    const R rm2 = R(1) / r2;
    const R rm6 = rm2 * rm2 * rm2;
    const R f = R(48.0) * rm2 * rm6 * (rm6 - R(0.5));
    return core ? f : lambda * f;
  }
  return R(0);
}

// FP32: 1/r2 as the correctly rounded reciprocal (the same bits as the
// division, without its general path)
template <>
__device__ __forceinline__ float pair_force<float>(int pot, bool bb, float r2, float lambda) {
  if (pot == POT_REF4824) {
    if (r2 < 1.0594631f || (bb && r2 < 2.25f)) {
      const float rm2 = __frcp_rn(r2);
      float rm24 = rm2 * rm2 * rm2;
      rm24 *= rm24;
      rm24 *= rm24;
      const float f = 192.0f * rm2 * rm24 * (rm24 - 0.5f);
      return r2 < 1.0594631f ? f : lambda * f;
    }
    return 0.0f;
  }
  if (r2 < 1.2599210498948732f || (bb && r2 < 6.25f)) {
    const float rm2 = __frcp_rn(r2);
    const float rm6 = rm2 * rm2 * rm2;
    const float f = 48.0f * rm2 * rm6 * (rm6 - 0.5f);
    return r2 < 1.2599210498948732f ? f : lambda * f;
  }
  return 0.0f;
}

template <typename R>
__device__ __forceinline__ R pair_pot(int pot, bool bb, R r2, R lambda) {
  if (pot == POT_REF4824) {
    if (r2 < R(1.0594631)) {
      R rm24 = R(1) / r2;
      rm24 *= rm24 * rm24;
      rm24 *= rm24;
      rm24 *= rm24;
      return R(4.0) * rm24 * (rm24 - R(1.0)) + R(1.0) - (bb ? lambda : R(0));
    }
    if (bb && r2 < R(2.25)) {
      R rm24 = R(1) / r2;
      rm24 *= rm24 * rm24;
      rm24 *= rm24;
      rm24 *= rm24;
      return R(4.0) * lambda * (rm24 * (rm24 - R(1.0)) - R(0.0000593));
    }
    return R(0);
  }
  if (r2 < R(1.2599210498948732) || (bb && r2 < R(6.25))) {
    R rm6 = R(1) / r2;
    rm6 *= rm6 * rm6;
    const R u = R(4.0) * rm6 * (rm6 - R(1.0));
    if (r2 < R(1.2599210498948732)) return u + R(1.0) - (bb ? lambda : R(0));
    return lambda * (u - R(-0.016316891136));
  }
  return R(0);
}

// Andersen stochastic thermostat of the MPC-off runs
// (AndersenStochastic::propagate, Thermostats/Andersen_stochastic.cpp:30-59):
// after the second half kick each bead, with probability nu dt, gets every
// velocity component drawn from N(0, sqrt(kT / m)). Draws: Philox on the
// replica's seed, counter (ANDERSEN_STREAM | bead, MD substep, k): k = 0 gives
// the trigger uniform and u1, k = 1 u2 and u3, k = 2 u4; Box-Muller pairs
// (u1, u2) -> x, y and (u3, u4) -> z.
constexpr uint32_t ANDERSEN_STREAM = 0x80000000u;

template <typename R>
__device__ __forceinline__ void andersen_draw(unsigned long long seed, int bead,
                                              unsigned long long md_step, R p, R sigma, R m,
                                              R* v) {
  const uint32_t c = ANDERSEN_STREAM | static_cast<uint32_t>(bead);
  const Uniform2<R> a = philox_uniforms<R>(seed, c, md_step, 0u);
  if (!(a.a < p)) return;
  const Uniform2<R> b = philox_uniforms<R>(seed, c, md_step, 1u);
  const Uniform2<R> d = philox_uniforms<R>(seed, c, md_step, 2u);
  const R two_pi = R(6.283185307179586476925286766559);
  const R s = sigma / r_sqrt(m);
  const R r1 = r_sqrt(R(-2) * r_log(a.b)), r2 = r_sqrt(R(-2) * r_log(b.b));
  R s1, c1, s2, c2;
  r_sincos(two_pi * b.a, &s1, &c1);
  r_sincos(two_pi * d.a, &s2, &c2);
  v[0] = s * (r1 * c1);
  v[1] = s * (r1 * s1);
  v[2] = s * (r2 * c2);
}

// FENE (Potentials.h:24-55): anchor bonds (core) use R0^2 = 20.25.
template <typename R>
__device__ __forceinline__ R fene_force(bool anchor, R r2) {
  return anchor ? R(-30.0) / (R(1.0) - (r2 / R(20.25))) : R(-30.0) / (R(1.0) - (r2 / R(2.25)));
}
template <>
__device__ __forceinline__ float fene_force<float>(bool anchor, float r2) {
  return -30.0f * __frcp_rn(1.0f - r2 * (anchor ? 1.0f / 20.25f : 1.0f / 2.25f));
}
template <typename R>
__device__ __forceinline__ R fene_pot(bool anchor, R r2) {
  return anchor ? R(-15.0) * R(20.25) * r_log(R(1.0) - r2 / R(20.25))
                : R(-15.0) * R(2.25) * r_log(R(1.0) - r2 / R(2.25));
}

struct MdArgs {
  const RepInfo* reps;
  RepDyn* dyn;
  const int* bond_start;   // CSR over global monomers
  const int2* bonds;       // (partner, anchor-bond flag)
  int* nlist;              // [max_nb][n_mono_total], transposed for coalescing
  int* ncount;             // [n_mono_total]
  int n_mono_total;
  int max_nb;
  int n_steps;             // substeps in this launch; 0 = build lists + forces only
  int calc_epot;
  int force_rebuild;
  int core_relative;       // fast path: displacements measured relative to the core's
  ErrorState* err;
  const int* order;        // replica of each CTA (largest first), or null: CTA b = replica b
  int andersen;            // Andersen stochastic thermostat (MPC-off runs)
  double andersen_nu;      // its collision frequency
  // Staged Andersen resets (smpc_stage_andersen), or null: replica r's
  // substep s resets beads and_mono[e] (replica-local) to and_vel[3 e ..] for
  // e in [and_start[r (n_steps + 1) + s], ... + s + 1); and_start[r (n_steps + 1)]
  // < 0 marks a replica that draws from Philox instead.
  const int* and_start;
  const int* and_mono;
  const double* and_vel;
  // Lowe-Andersen pair thermostat (MPC-off runs): collision frequency in
  // andersen_nu, interaction radius, scratch of LOWE_MAX LoweEntry<R> per
  // monomer (null when off)
  int lowe;
  double lowe_radius;
  void* lowe_buf;
};

// Lowe-Andersen thermostat (Lowe_Andersen::propagate, Thermostats/
// Lowe_Andersen.cpp:46-88): after the forces of a substep and before its
// second half kick, every Verlet-list entry (i, j) is a collision candidate
// with probability NuDt / 2, NuDt = nu dt exp(-nu dt); a candidate closer than
// the interaction radius exchanges momentum along the pair axis e:
//   dv = e (sqrt(kT / mu) z + (v_j - v_i) . e),  v_i += dv mu / m_i,  v_j -= dv mu / m_j,
// mu the reduced mass (m / 2 for equal masses), z a standard normal.
// Collisions act one after another on the updated velocities, so their order
// is part of the result: here it is canonical, beads i ascending and each
// bead's partners j ascending (the reference walks its lists in the order its
// cell lists produce). Draws: Philox on the replica's seed, counter
// (LOWE_STREAM | i, MD substep, 2 j + k): k = 0 gives the trigger uniform and
// u1, k = 1 gives u2; z = sqrt(-2 ln u1) cos(2 pi u2).
constexpr uint32_t LOWE_STREAM = 0x40000000u;
constexpr int LOWE_MAX = 16;  // accepted collisions per bead and substep (an error beyond)

template <typename R>
struct LoweEntry {
  int i, j;
  R e0, e1, e2;  // unit pair axis, from i to j
  R tv;          // sqrt(kT / mu) z
  R ci, cj;      // mu / m_i, mu / m_j
};

// One substep's collisions of the replica at monomer base b (n beads), run by
// the whole CTA: candidates by each bead's lead lane, offsets by warp 0, the
// velocity updates in canonical order by thread 0 on velocities staged in
// sx/sy/sz (the positions there are not needed again before the next drift
// rewrites them). v[k] of every lane comes back updated.
template <typename R, int NT, int MPT>
__device__ void lowe_andersen_pass(const MdArgs& a, const RepInfo& ri, int b, int n, int slot,
                                   bool lead, unsigned long long md_step, const R (&x)[MPT][3],
                                   R (&v)[MPT][3], const R (&m)[MPT], const R* mpos, R* sx, R* sy,
                                   R* sz, int* s_cnt, int* s_off, int* s_total) {
  LoweEntry<R>* buf = static_cast<LoweEntry<R>*>(a.lowe_buf) + static_cast<size_t>(b) * LOWE_MAX;
  const double nudt = a.andersen_nu * ri.md_dt * exp(-ri.md_dt * a.andersen_nu);
  const R half = static_cast<R>(nudt * 0.5);
  const R radius = static_cast<R>(a.lowe_radius);
  const R kT = static_cast<R>(ri.kT);
  const size_t stride = static_cast<size_t>(a.n_mono_total);
  int acc[MPT][LOWE_MAX];
  int na[MPT];
  __syncthreads();  // the forces are done with sx/sy/sz
#pragma unroll
  for (int k = 0; k < MPT; ++k) {
    const int i = slot + k * NT;
    na[k] = 0;
    if (i >= n || !lead) continue;
    const int cnt = a.ncount[b + i];
    for (int q = 0; q < cnt; ++q) {
      const int j = a.nlist[static_cast<size_t>(q) * stride + b + i] - b;
      const Uniform2<R> t = philox_uniforms<R>(ri.seed, LOWE_STREAM | static_cast<uint32_t>(i),
                                               md_step, 2u * static_cast<uint32_t>(j));
      if (half < t.a) continue;  // Lowe_Andersen.cpp:71
      const R d0 = sx[j] - x[k][0], d1 = sy[j] - x[k][1], d2 = sz[j] - x[k][2];
      if (!(r_sqrt((d0 * d0 + d1 * d1) + d2 * d2) < radius)) continue;  // Lowe_Andersen.cpp:31
      if (na[k] < LOWE_MAX) {
        int p = na[k];
        while (p > 0 && acc[k][p - 1] > j) {
          acc[k][p] = acc[k][p - 1];
          --p;
        }
        acc[k][p] = j;
      } else {
        raise_error(a.err, ERR_NEIGHBOR_OVF, static_cast<uint32_t>(b + i), LOWE_MAX + 1u);
      }
      ++na[k];
    }
    if (na[k] > LOWE_MAX) na[k] = LOWE_MAX;
    s_cnt[i] = na[k];
  }
  __syncthreads();
  if (threadIdx.x < 32) {  // exclusive offsets of the beads' collisions
    const int lane = threadIdx.x;
    int carry = 0;
    for (int base = 0; base < n; base += 32) {
      const int i = base + lane;
      const int c = i < n ? s_cnt[i] : 0;
      int incl = c;
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += t;
      }
      if (i < n) s_off[i] = carry + incl - c;
      carry += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) *s_total = carry;
  }
  __syncthreads();
  const R two_pi = R(6.283185307179586476925286766559);
#pragma unroll
  for (int k = 0; k < MPT; ++k) {
    const int i = slot + k * NT;
    if (i >= n || !lead) continue;
    for (int q = 0; q < na[k]; ++q) {
      const int j = acc[k][q];
      const R d0 = sx[j] - x[k][0], d1 = sy[j] - x[k][1], d2 = sz[j] - x[k][2];
      const R dist = r_sqrt((d0 * d0 + d1 * d1) + d2 * d2);
      const R mi = m[k], mj = mpos[4 * static_cast<size_t>(b + j) + 3];
      const R mu = mi == mj ? R(0.5) * mi : mi * mj / (mi + mj);
      const R sigma = r_sqrt(kT / mu);
      const uint32_t c = LOWE_STREAM | static_cast<uint32_t>(i);
      const Uniform2<R> t0 = philox_uniforms<R>(ri.seed, c, md_step, 2u * static_cast<uint32_t>(j));
      const Uniform2<R> t1 =
          philox_uniforms<R>(ri.seed, c, md_step, 2u * static_cast<uint32_t>(j) + 1u);
      const R z = r_sqrt(R(-2) * r_log(t0.b)) * r_cos(two_pi * t1.a);
      LoweEntry<R> e;
      e.i = i;
      e.j = j;
      e.e0 = d0 / dist;
      e.e1 = d1 / dist;
      e.e2 = d2 / dist;
      e.tv = sigma * z;
      e.ci = mu / mi;
      e.cj = mu / mj;
      buf[s_off[i] + q] = e;
    }
  }
  __syncthreads();  // entries written, positions no longer read
#pragma unroll
  for (int k = 0; k < MPT; ++k) {
    const int i = slot + k * NT;
    if (i < n && lead) {
      sx[i] = v[k][0];
      sy[i] = v[k][1];
      sz[i] = v[k][2];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int total = *s_total;
    for (int q = 0; q < total; ++q) {
      const LoweEntry<R> e = buf[q];
      const R w0 = sx[e.j] - sx[e.i], w1 = sy[e.j] - sy[e.i], w2 = sz[e.j] - sz[e.i];
      const R sc = e.tv + ((w0 * e.e0 + w1 * e.e1) + w2 * e.e2);
      const R dv0 = e.e0 * sc, dv1 = e.e1 * sc, dv2 = e.e2 * sc;
      sx[e.i] += dv0 * e.ci;
      sy[e.i] += dv1 * e.ci;
      sz[e.i] += dv2 * e.ci;
      sx[e.j] -= dv0 * e.cj;
      sy[e.j] -= dv1 * e.cj;
      sz[e.j] -= dv2 * e.cj;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < MPT; ++k) {
    const int i = slot + k * NT;
    if (i < n) {
      v[k][0] = sx[i];
      v[k][1] = sy[i];
      v[k][2] = sz[i];
    }
  }
}

// Cell key of a position on a grid of side rv: three 10-bit fields
// (coordinates within +-512 cells of the origin) and a bucket hash.
constexpr int MD_BUCKETS = 2048;
__device__ __forceinline__ int md_cell_key(int cx, int cy, int cz) {
  return ((cx + 512) & 1023) | (((cy + 512) & 1023) << 10) | (((cz + 512) & 1023) << 20);
}
__device__ __forceinline__ int md_bucket(int cx, int cy, int cz) {
  return static_cast<int>((static_cast<unsigned>(cx) * 73856093u) ^
                          (static_cast<unsigned>(cy) * 19349663u) ^
                          (static_cast<unsigned>(cz) * 83492791u)) &
         (MD_BUCKETS - 1);
}

// inclusive warp scan
__device__ __forceinline__ int md_warp_scan(int v) {
  const int lane = static_cast<int>(threadIdx.x & 31u);
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Beads in bucket order, each bucket in ascending bead order (the order the
// sorted chains give), as a counting sort: one warp ranks the beads within
// their buckets in bead order, 32 at a time (__match_any_sync groups a
// batch's beads by bucket), the block scans the counts, and every bead goes
// to its bucket's start plus its rank. s_bkt[j]: bucket of bead j, set by
// the caller (the rank is packed beside it: bucket | rank << 11);
// s_start[MD_BUCKETS + 1]: bucket starts; s_sorted[k]: the k-th bead. Ends
// with the block synchronised. A cell's members are then a contiguous run to
// scan, not a chain of dependent loads.
template <int NT>
__device__ __forceinline__ void md_bucket_sort(int n, int* s_bkt, int* s_start, int* s_sorted) {
  static_assert(MD_BUCKETS == 2048, "11-bit bucket field");
  static_assert(MD_BUCKETS % NT == 0 && NT % 32 == 0, "bucket scan layout");
  constexpr int PER = MD_BUCKETS / NT;
  for (int t = threadIdx.x; t <= MD_BUCKETS; t += NT) s_start[t] = 0;
  __syncthreads();
  if (threadIdx.x < 32) {
    const unsigned lane = threadIdx.x;
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + static_cast<int>(lane);
      const int bk = j < n ? s_bkt[j] : -1 - static_cast<int>(lane);
      const unsigned peers = __match_any_sync(0xFFFFFFFFu, bk);
      const int leader = __ffs(peers) - 1;
      int base = 0;
      if (j < n && static_cast<int>(lane) == leader) {
        base = s_start[bk];
        s_start[bk] = base + __popc(peers);
      }
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (j < n) s_bkt[j] = bk | ((base + __popc(peers & ((1u << lane) - 1u))) << 11);
    }
  }
  __syncthreads();
  {  // exclusive scan of the counts: PER consecutive buckets per thread
    __shared__ int s_wsum[NT / 32];
    int c[PER], tot = 0;
#pragma unroll
    for (int u = 0; u < PER; ++u) { c[u] = s_start[PER * threadIdx.x + u]; tot += c[u]; }
    const int inc = md_warp_scan(tot);
    if ((threadIdx.x & 31u) == 31u) s_wsum[threadIdx.x >> 5] = inc;
    __syncthreads();
    int wbase = 0;
    for (int w = 0; w < static_cast<int>(threadIdx.x >> 5); ++w) wbase += s_wsum[w];
    int run = wbase + inc - tot;
#pragma unroll
    for (int u = 0; u < PER; ++u) { s_start[PER * threadIdx.x + u] = run; run += c[u]; }
    if (threadIdx.x == NT - 1) s_start[MD_BUCKETS] = run;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += NT)
    s_sorted[s_start[s_bkt[j] & 2047] + (s_bkt[j] >> 11)] = j;
  __syncthreads();
}

// The 512-thread lanes-per-bead shape is held to 64 registers so that two of
// its blocks share an SM (the side-by-side MD launch shape).
template <typename R, int NT, int MPT, int KMAX = 1>
__global__ void __launch_bounds__(NT, (NT == 512 && KMAX > 1) ? 2 : 1)
    k_md_substeps(MdArgs a, R* mpos, R* mvel, R* mfrc, R* mver) {
  static_assert(KMAX == 1 || MPT == 1, "lanes per bead > 1 needs one bead per thread");
  constexpr int CAP = NT * MPT;
  __shared__ R sx[CAP], sy[CAP], sz[CAP];
  __shared__ unsigned char s_amphi[CAP];
  __shared__ int s_head[MD_BUCKETS + 1];  // bucket starts in s_sorted
  __shared__ int s_next[CAP];             // bucket of each bead
  __shared__ int s_ckey[CAP];
  __shared__ int s_sorted[CAP];
  __shared__ R s_core_ref[3];
  __shared__ int s_rebuild;
  __shared__ int s_lowe_total;
  __shared__ double s_red[NT / 32];
  const int r = a.order ? a.order[blockIdx.x] : static_cast<int>(blockIdx.x);
  const RepInfo ri = a.reps[r];
  const int n = ri.n_mono;
  if (n == 0 || (ri.flags & REP_PERIODIC_MD)) return;  // periodic boxes: pmd_kernels.cuh
  int lk = 0;  // log2 of the lanes per bead
  if (KMAX > 1)
    while ((2 << lk) <= KMAX && (n << (lk + 1)) <= NT) ++lk;
  const int sub = static_cast<int>(threadIdx.x) & ((1 << lk) - 1);
  const int slot = static_cast<int>(threadIdx.x) >> lk;  // bead of this lane (k = 0)
  const bool lead = sub == 0;
  const int b = ri.mono_base;
  const R dt = static_cast<R>(ri.md_dt);
  const R dth = dt * R(0.50);
  const R lambda = static_cast<R>(ri.lambda);
  const R rv2 = static_cast<R>(ri.r_verlet) * static_cast<R>(ri.r_verlet);
  const R lim = (static_cast<R>(ri.r_verlet) - static_cast<R>(ri.r_cut)) * R(0.5);
  const int pot = ri.potential;
  const unsigned long long md_step0 = a.dyn[r].md_step;  // thread 0 adds n_steps at the end

  R x[MPT][3], v[MPT][3], f[MPT][3], xv[MPT][3], m[MPT];
  int anc[MPT];
#pragma unroll
  for (int k = 0; k < MPT; ++k) {
    const int i = slot + k * NT;
    if (i < n) {
      const R4<R> p = ld4_rw(mpos, b + i), vv = ld4_rw(mvel, b + i), ff = ld4_rw(mfrc, b + i),
                  pv = ld4_rw(mver, b + i);
      x[k][0] = p.x; x[k][1] = p.y; x[k][2] = p.z; m[k] = p.w;
      v[k][0] = vv.x; v[k][1] = vv.y; v[k][2] = vv.z;
      const int flags = static_cast<int>(vv.w);
      anc[k] = (flags >> 1) & 1;
      f[k][0] = ff.x; f[k][1] = ff.y; f[k][2] = ff.z;
      xv[k][0] = pv.x; xv[k][1] = pv.y; xv[k][2] = pv.z;
      if (lead) {
        s_amphi[i] = static_cast<unsigned char>(flags & 1);
        sx[i] = p.x; sy[i] = p.y; sz[i] = p.z;
      }
    }
  }
  if (threadIdx.x == 0) {
    s_rebuild = a.force_rebuild;
    // the core's position at the last list build (its Verlet reference)
    const R4<R> c = ld4_rw(mver, b);
    s_core_ref[0] = c.x; s_core_ref[1] = c.y; s_core_ref[2] = c.z;
  }
  __syncthreads();
  int rebuilds = 0;
  double epot = 0.0;
  const int total_steps = a.n_steps > 0 ? a.n_steps : 1;
  for (int step = 0; step < total_steps; ++step) {
    if (a.n_steps > 0) {
      // kick + drift (Thermostat_None.cpp:22-27)
#pragma unroll
      for (int k = 0; k < MPT; ++k) {
        const int i = slot + k * NT;
        if (i < n) {
          for (int d = 0; d < 3; ++d) {
            v[k][d] += a.andersen ? f[k][d] * (dth / m[k]) : (f[k][d] / m[k]) * dth;
            x[k][d] += v[k][d] * dt;
          }
          if (lead) { sx[i] = x[k][0]; sy[i] = x[k][1]; sz[i] = x[k][2]; }
          if (!a.core_relative) {
            // Box::check_VerletLists (Box.cpp:182-194)
            const R d0 = x[k][0] - xv[k][0], d1 = x[k][1] - xv[k][1], d2 = x[k][2] - xv[k][2];
            if (r_sqrt((d0 * d0 + d1 * d1) + d2 * d2) > lim) s_rebuild = 1;
          }
        }
      }
      if (a.core_relative) {
        // Pair distances change by at most |dr_i - c| + |dr_j - c| for any
        // common c; with c the core's displacement, a star carried by the
        // flow does not trigger rebuilds.
        __syncthreads();
        const R c0 = sx[0] - s_core_ref[0], c1 = sy[0] - s_core_ref[1], c2 = sz[0] - s_core_ref[2];
#pragma unroll
        for (int k = 0; k < MPT; ++k) {
          const int i = slot + k * NT;
          if (i < n) {
            const R d0 = x[k][0] - xv[k][0] - c0, d1 = x[k][1] - xv[k][1] - c1,
                    d2 = x[k][2] - xv[k][2] - c2;
            if ((d0 * d0 + d1 * d1) + d2 * d2 > lim * lim) s_rebuild = 1;
          }
        }
      }
    }
    __syncthreads();
    const int rebuild = s_rebuild;
    if (rebuild) {
      // Verlet lists: every other bead within r_verlet (Box.cpp:146-179), found
      // through a hashed grid of side r_verlet in shared memory
      ++rebuilds;
      const R inv_rv = R(1) / static_cast<R>(ri.r_verlet);
      int cx[MPT], cy[MPT], cz[MPT];
#pragma unroll
      for (int k = 0; k < MPT; ++k) {
        const int i = slot + k * NT;
        if (i < n) {
          cx[k] = static_cast<int>(floor(x[k][0] * inv_rv));
          cy[k] = static_cast<int>(floor(x[k][1] * inv_rv));
          cz[k] = static_cast<int>(floor(x[k][2] * inv_rv));
          if (lead) {
            s_ckey[i] = md_cell_key(cx[k], cy[k], cz[k]);
            s_next[i] = md_bucket(cx[k], cy[k], cz[k]);
          }
        }
      }
      __syncthreads();
      md_bucket_sort<NT>(n, s_next, s_head, s_sorted);
#pragma unroll
      for (int k = 0; k < MPT; ++k) {
        const int i = slot + k * NT;
        if (i < n && lead) {
          int cnt = 0;
          for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dx = -1; dx <= 1; ++dx) {
                const int tx = cx[k] + dx, ty = cy[k] + dy, tz = cz[k] + dz;
                const int want = md_cell_key(tx, ty, tz);
                const int bk = md_bucket(tx, ty, tz);
                const int kend = s_head[bk + 1];
                for (int kk = s_head[bk]; kk < kend; ++kk) {
                  const int j = s_sorted[kk];
                  if (j == i || s_ckey[j] != want) continue;
                  const R d0 = sx[j] - x[k][0], d1 = sy[j] - x[k][1], d2 = sz[j] - x[k][2];
                  if ((d0 * d0 + d1 * d1) + d2 * d2 <= rv2) {
                    if (cnt < a.max_nb)
                      a.nlist[static_cast<size_t>(cnt) * a.n_mono_total + b + i] = b + j;
                    ++cnt;
                  }
                }
              }
          if (cnt > a.max_nb) {
            raise_error(a.err, ERR_NEIGHBOR_OVF, static_cast<uint32_t>(b + i),
                        static_cast<uint32_t>(cnt));
            cnt = a.max_nb;
          }
          a.ncount[b + i] = cnt;
        }
        if (i < n) { xv[k][0] = x[k][0]; xv[k][1] = x[k][1]; xv[k][2] = x[k][2]; }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        s_core_ref[0] = sx[0]; s_core_ref[1] = sy[0]; s_core_ref[2] = sz[0];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) s_rebuild = 0;
    const bool want_epot = a.calc_epot && (step == total_steps - 1);
    // forces (Box.cpp:243-286)
#pragma unroll
    for (int k = 0; k < MPT; ++k) {
      const int i = slot + k * NT;
      R F0 = R(0), F1 = R(0), F2 = R(0);
      if (i < n) {
        const bool ai = s_amphi[i] != 0;
        const int cnt = a.ncount[b + i];
        const int* nl = a.nlist + b + i;
        const size_t stride = static_cast<size_t>(a.n_mono_total);
        // neighbour indices come in groups of four independent loads, so the
        // list walk is not a chain of dependent L2 round trips; the lanes of
        // a bead take every (1 << lk)-th entry
        constexpr int PF = 4;
        for (int q0 = sub; q0 < cnt; q0 += PF << lk) {
          int js[PF];
#pragma unroll
          for (int u = 0; u < PF; ++u) {
            const int q = q0 + (u << lk);
            js[u] = q < cnt ? nl[static_cast<size_t>(q) * stride] - b : -1;
          }
#pragma unroll
          for (int u = 0; u < PF; ++u) {
            const int j = js[u];
            if (j < 0) continue;
            const R d0 = sx[j] - x[k][0], d1 = sy[j] - x[k][1], d2 = sz[j] - x[k][2];
            const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
            const bool bb = ai && s_amphi[j] != 0;
            const R fa = pair_force<R>(pot, bb, r2, lambda);
            F0 -= d0 * fa;
            F1 -= d1 * fa;
            F2 -= d2 * fa;
            if (want_epot) epot += 0.5 * static_cast<double>(pair_pot<R>(pot, bb, r2, lambda));
          }
        }
        for (int e = lead ? a.bond_start[b + i] : 0; lead && e < a.bond_start[b + i + 1]; ++e) {
          const int2 bd = a.bonds[e];
          const int j = bd.x - b;
          const R d0 = sx[j] - x[k][0], d1 = sy[j] - x[k][1], d2 = sz[j] - x[k][2];
          const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
          const bool anch = bd.y != 0;
          R r2f = r2;
          if (pot == POT_REF4824) {
            // reference FENE: beyond R0 the force changes sign (Potentials.h:24-55)
            if (r2 >= (anch ? R(20.25) : R(2.25)))
              raise_error(a.err, ERR_FENE, static_cast<uint32_t>(b + i), static_cast<uint32_t>(b + j));
          } else {
            // 12-6 preset: FENE argument capped at 0.98 R0^2 (finite, restoring)
            const R cap = (anch ? R(20.25) : R(2.25)) * R(0.98);
            if (r2f > cap) r2f = cap;
          }
          const R fa = fene_force<R>(anch, r2f);
          F0 -= d0 * fa;
          F1 -= d1 * fa;
          F2 -= d2 * fa;
          if (want_epot) epot += 0.5 * static_cast<double>(fene_pot<R>(anch, r2f));
        }
      }
      // partial forces of a bead's lanes (every lane of the warp takes part)
      for (int o = 1; KMAX > 1 && o < (1 << lk); o <<= 1) {
        F0 += __shfl_xor_sync(0xFFFFFFFFu, F0, o);
        F1 += __shfl_xor_sync(0xFFFFFFFFu, F1, o);
        F2 += __shfl_xor_sync(0xFFFFFFFFu, F2, o);
      }
      if (i < n) {
        f[k][0] = F0; f[k][1] = F1; f[k][2] = F2;
        if (a.n_steps > 0 && !a.lowe) {
          for (int d = 0; d < 3; ++d)  // second half-kick
            v[k][d] += a.andersen ? f[k][d] * (dth / m[k]) : (f[k][d] / m[k]) * dth;
          if (a.andersen) {
            const int* as = a.and_start ? a.and_start + static_cast<size_t>(r) * (a.n_steps + 1)
                                        : nullptr;
            if (as && as[0] >= 0) {
              for (int e = as[step]; e < as[step + 1]; ++e)
                if (a.and_mono[e] == i)
                  for (int d = 0; d < 3; ++d) v[k][d] = static_cast<R>(a.and_vel[3 * e + d]);
            } else {
              andersen_draw<R>(ri.seed, i, md_step0 + static_cast<unsigned long long>(step),
                               static_cast<R>(a.andersen_nu * ri.md_dt),
                               r_sqrt(static_cast<R>(ri.kT)), m[k], v[k]);
            }
          }
        }
      }
    }
    if (a.lowe && a.n_steps > 0) {
      // pair collisions between the forces and the second half kick
      lowe_andersen_pass<R, NT, MPT>(a, ri, b, n, slot, lead,
                                     md_step0 + static_cast<unsigned long long>(step), x, v, m,
                                     mpos, sx, sy, sz, s_next, s_ckey, &s_lowe_total);
#pragma unroll
      for (int k = 0; k < MPT; ++k) {
        const int i = slot + k * NT;
        if (i < n)
          for (int d = 0; d < 3; ++d) v[k][d] += (f[k][d] / m[k]) * dth;
      }
    }
    __syncthreads();  // positions are rewritten by the next drift
  }
  // write back
#pragma unroll
  for (int k = 0; k < MPT; ++k) {
    const int i = slot + k * NT;
    if (i < n && lead) {
      R4<R> p = ld4_rw(mpos, b + i);
      p.x = x[k][0]; p.y = x[k][1]; p.z = x[k][2];
      st4(mpos, b + i, p);
      R4<R> vv = ld4_rw(mvel, b + i);
      vv.x = v[k][0]; vv.y = v[k][1]; vv.z = v[k][2];
      st4(mvel, b + i, vv);
      st4(mfrc, b + i, R4<R>{f[k][0], f[k][1], f[k][2], R(0)});
      st4(mver, b + i, R4<R>{xv[k][0], xv[k][1], xv[k][2], R(0)});
    }
  }
  if (a.calc_epot) {
    for (int o = 16; o > 0; o >>= 1) epot += __shfl_down_sync(0xFFFFFFFFu, epot, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = epot;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < NT / 32; ++w) s += s_red[w];
      a.dyn[r].epot = s;
    }
  }
  if (threadIdx.x == 0) {
    a.dyn[r].verlet_rebuilds += rebuilds;
    if (a.n_steps > 0) a.dyn[r].md_step = md_step0 + static_cast<unsigned long long>(a.n_steps);
  }
}

// Paths of k_md_cluster that most substeps do not take, out of line, so that
// the code of a substep stays compact: half the pair and FENE energies (read
// at the last substep of a call when asked for), the Andersen resets, and the
// lanes-per-bead force walk over the global lists (a CTA whose lists outgrow
// the shared buffers).
template <typename R>
__device__ __noinline__ double md_pair_epot(int pot, bool bb, R r2, R lambda) {
  return 0.5 * static_cast<double>(pair_pot<R>(pot, bb, r2, lambda));
}
template <typename R>
__device__ __noinline__ double md_fene_epot(bool anch, R r2) {
  return 0.5 * static_cast<double>(fene_pot<R>(anch, r2));
}
template <typename R>
__device__ __noinline__ void md_andersen_reset(const MdArgs& a, const RepInfo& ri, int r, int step,
                                               int ik, unsigned long long md_step0, R m, R* v) {
  const int* as = a.and_start ? a.and_start + static_cast<size_t>(r) * (a.n_steps + 1) : nullptr;
  if (as && as[0] >= 0) {
    for (int e = as[step]; e < as[step + 1]; ++e)
      if (a.and_mono[e] == ik)
        for (int d = 0; d < 3; ++d) v[d] = static_cast<R>(a.and_vel[3 * e + d]);
  } else {
    andersen_draw<R>(ri.seed, ik, md_step0 + static_cast<unsigned long long>(step),
                     static_cast<R>(a.andersen_nu * ri.md_dt), r_sqrt(static_cast<R>(ri.kT)), m, v);
  }
}
// Forces on bead i (replica-local; mono_base b) from its Verlet list in global
// memory, every (1 << lk)-th entry from sub, and its bonds on the lead lane;
// F accumulates them, epot (when asked) half the energies.
template <typename R>
__device__ __noinline__ void md_bead_forces_lists(const MdArgs& a, int b, int i, int sub, int lk,
                                                  bool lead, const R* sx, const R* sy,
                                                  const R* sz, const unsigned char* s_amphi,
                                                  int pot, R lambda, bool want_epot, R* F,
                                                  double* epot) {
  const R x0 = sx[i], x1 = sy[i], x2 = sz[i];
  R F0 = F[0], F1 = F[1], F2 = F[2];
  const bool ai = s_amphi[i] != 0;
  const int cnt = a.ncount[b + i];
  const int* nl = a.nlist + b + i;
  const size_t stride = static_cast<size_t>(a.n_mono_total);
  constexpr int PF = 4;
  for (int q0 = sub; q0 < cnt; q0 += PF << lk) {
    int js[PF];
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int qq = q0 + (u << lk);
      js[u] = qq < cnt ? nl[static_cast<size_t>(qq) * stride] - b : -1;
    }
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int j = js[u];
      if (j < 0) continue;
      const R d0 = sx[j] - x0, d1 = sy[j] - x1, d2 = sz[j] - x2;
      const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
      const bool bb = ai && s_amphi[j] != 0;
      const R fa = pair_force<R>(pot, bb, r2, lambda);
      F0 -= d0 * fa;
      F1 -= d1 * fa;
      F2 -= d2 * fa;
      if (want_epot) *epot += md_pair_epot<R>(pot, bb, r2, lambda);
    }
  }
  for (int e = lead ? a.bond_start[b + i] : 0; lead && e < a.bond_start[b + i + 1]; ++e) {
    const int2 bd = a.bonds[e];
    const int j = bd.x - b;
    const R d0 = sx[j] - x0, d1 = sy[j] - x1, d2 = sz[j] - x2;
    const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
    const bool anch = bd.y != 0;
    R r2f = r2;
    if (pot == POT_REF4824) {
      if (r2 >= (anch ? R(20.25) : R(2.25)))
        raise_error(a.err, ERR_FENE, static_cast<uint32_t>(b + i), static_cast<uint32_t>(b + j));
    } else {
      const R cap = (anch ? R(20.25) : R(2.25)) * R(0.98);
      if (r2f > cap) r2f = cap;
    }
    const R fa = fene_force<R>(anch, r2f);
    F0 -= d0 * fa;
    F1 -= d1 * fa;
    F2 -= d2 * fa;
    if (want_epot) *epot += md_fene_epot<R>(anch, r2f);
  }
  F[0] = F0;
  F[1] = F1;
  F[2] = F2;
}


// ---------------------------------------------------------------------------
// The same substeps for one replica on a thread-block cluster of CS CTAs (CS
// SMs), for boxes with few replicas: one CTA's FP64 pipe (2 DFMA per clock
// per SM on this part) held a 401-bead star's FP64 MD to 150 us per substep.
// Every CTA keeps a copy of all positions in its shared memory and owns the
// beads i = rank + CS q. After the drift each CTA's beads go into its own
// copy, then into every other CTA's (distributed shared memory, one (bead,
// CTA) pair per thread); a bead past the Verlet limit sets every CTA's
// rebuild flag. The copies are double-buffered by substep parity, so one
// cluster barrier per substep, after the drift, suffices (positions and
// flags complete everywhere); with displacements measured relative to the
// core, every CTA decides the rebuild for all beads itself. A rebuild hashes
// all beads in every CTA's own grid; each CTA writes the lists of its own
// beads. Forces, kicks and the Andersen resets are those of k_md_substeps
// for the owned beads. The barriers are hardware cluster barriers: every CTA
// of a cluster runs at once, and every CTA reaches every barrier (no branch
// around one). Lowe-Andersen stays on k_md_substeps.
// The kicks and the drift of a CTA's beads run one thread per bead (threads
// 0 .. own-1, in whole warps), not on the lead lane of each bead's lanes: on
// the narrow FP64 pipe a warp instruction costs the same with one active
// lane as with 32. Forces reach those threads through shared memory.
//
// Pair forces are compacted. Most Verlet-list entries lie beyond the
// interaction range, and with lanes per bead walking the lists a warp issued
// each FP64 force instruction for the few lanes whose pair was in range (7.7
// active lanes per instruction). Instead, the CTA keeps its beads' lists
// flattened in shared memory (bead by bead, each in list order), and per
// substep:
//  1. every warp tests a contiguous run of entries in FP32 (positions kept
//     in FP32 beside the FP64 copy) against the pair's cut-off widened by
//     2^-7, and writes the entries that pass into a candidate list by ballot
//     (the list stays in flattened order);
//  2. all threads compute the candidates' FP64 pair forces, every lane busy,
//     with the exact FP64 range test inside pair_force, and the bonds' FENE
//     forces, one bond per thread;
//  3. each bead's lanes subtract its pairs' contributions, lane l taking
//     every lanes-th one from the l-th, then its bonds' the same way, and
//     sum over the lanes (Box.cpp:253-284 subtracts them one by one; the
//     order here is fixed, so runs repeat bit for bit).
// The FP32 test only skips entries whose FP64 force is zero: FP32 rounding
// of coordinates below 4096 moves r^2 by far less than the margin. A CTA whose
// lists or bonds outgrow the shared buffers, or a replica with a coordinate
// of 4096 or more, takes the lanes-per-bead pass instead.
constexpr int MD_CLUSTER_CAP = 1024;
constexpr int MDC_ECAP = 8192;  // flattened list entries of a CTA's beads
constexpr int MDC_CCAP = 1024;  // candidate pairs per force batch
constexpr int MDC_BCAP = 512;   // bonds of a CTA's beads
constexpr float MDC_FAR = 4096.0f;

// Dynamic shared memory of k_md_cluster<R, NT, CS, KMAX> (byte offsets).
template <typename R, int CS>
struct MdcLayout {
  static constexpr int OWN = (MD_CLUSTER_CAP + CS - 1) / CS;  // beads per CTA at most
  static constexpr size_t posr = 0;                                    // R[2][3][CAP] positions
  // float[2][3][CAP], FP64 only
  static constexpr size_t posf = posr + sizeof(R) * 6 * MD_CLUSTER_CAP;
  static constexpr size_t xvf = posf + (sizeof(R) == 8 ? sizeof(float) * 6 * MD_CLUSTER_CAP : 0);
  static constexpr size_t pf = xvf + sizeof(float) * 3 * MD_CLUSTER_CAP;  // R[3 CCAP]
  static constexpr size_t bf = pf + sizeof(R) * 3 * MDC_CCAP;          // R[3 BCAP]
  static constexpr size_t cand = bf + sizeof(R) * 3 * MDC_BCAP;        // int[ECAP]
  static constexpr size_t bj = cand + sizeof(int) * MDC_ECAP;          // int[BCAP]
  static constexpr size_t lstart = bj + sizeof(int) * MDC_BCAP;        // int[OWN + 1]
  static constexpr size_t cstart = lstart + sizeof(int) * (OWN + 1);   // int[OWN + 1]
  static constexpr size_t bstart = cstart + sizeof(int) * (OWN + 1);   // int[OWN + 1]
  static constexpr size_t nb = bstart + sizeof(int) * (OWN + 1);       // uint16[ECAP]
  static constexpr size_t own = nb + 2 * MDC_ECAP;                     // uint8[ECAP]
  static constexpr size_t bq = own + MDC_ECAP;                         // uint8[BCAP]
  static constexpr size_t bytes = bq + MDC_BCAP;
  static_assert(OWN <= 256, "bead slot of a CTA fits one byte");
};


template <typename R, int NT, int CS, int KMAX>
__global__ void __launch_bounds__(NT, 1) k_md_cluster(MdArgs a, R* mpos, R* mvel, R* mfrc, R* mver) {
  namespace cg = cooperative_groups;
  constexpr int CAP = MD_CLUSTER_CAP;
  __shared__ unsigned char s_amphi[CAP];
  __shared__ int s_head[MD_BUCKETS + 1];  // bucket starts in s_sorted
  __shared__ int s_next[CAP];             // bucket of each bead
  __shared__ int s_ckey[CAP];
  __shared__ int s_sorted[CAP];
  __shared__ float s_coref[3];      // the core's position at the last rebuild (FP32)
  __shared__ int s_rebuild[2];      // by substep parity: a bead passed the Verlet limit
  __shared__ int s_farp[2];         // by substep parity: a coordinate reached MDC_FAR
  __shared__ double s_red[NT / 32];
  __shared__ double s_epot[CS];
  __shared__ R s_f[3 * ((CAP + CS - 1) / CS)];  // forces of this CTA's beads
  static_assert((CAP + CS - 1) / CS <= NT, "a kick thread for every bead of the CTA");
  constexpr int NW = NT / 32;
  static_assert((NW & (NW - 1)) == 0, "a power of two of warps (candidate search)");
  constexpr bool kF64 = sizeof(R) == 8;
  using L = MdcLayout<R, CS>;
  __shared__ int s_wcnt[NW], s_woff[NW + 1];
  // per warp and round of 32 list entries: candidates before the round, and
  // the round's ballot of candidates (list position -> candidate position)
  constexpr int MDC_ROUNDS = (MDC_ECAP / NW + 31) / 32;
  __shared__ int s_rpre[MDC_ROUNDS][NW];
  __shared__ unsigned s_rmask[MDC_ROUNDS][NW];
  __shared__ int s_far, s_fits;  // replica-wide: a coordinate >= MDC_FAR so far; CTA: lists fit
  extern __shared__ __align__(16) unsigned char s_dyn[];
  // Positions, double-buffered by substep parity: substep s pushes into and
  // reads from buffer s & 1, so one cluster barrier per substep suffices (a
  // CTA pushing substep s + 1 has passed the barrier of substep s, which
  // every CTA reached after its last read of buffer (s + 1) & 1).
  R* const s_posr = reinterpret_cast<R*>(s_dyn + L::posr);
  float* const s_posf = reinterpret_cast<float*>(s_dyn + L::posf);
  float* const s_xvf = reinterpret_cast<float*>(s_dyn + L::xvf);  // Verlet reference positions
  R* s_pf = reinterpret_cast<R*>(s_dyn + L::pf);
  R* s_bf = reinterpret_cast<R*>(s_dyn + L::bf);
  int* s_cand = reinterpret_cast<int*>(s_dyn + L::cand);
  int* s_bj = reinterpret_cast<int*>(s_dyn + L::bj);
  int* s_lstart = reinterpret_cast<int*>(s_dyn + L::lstart);
  int* s_cstart = reinterpret_cast<int*>(s_dyn + L::cstart);
  int* s_bstart = reinterpret_cast<int*>(s_dyn + L::bstart);
  unsigned short* s_nb = reinterpret_cast<unsigned short*>(s_dyn + L::nb);
  unsigned char* s_own = s_dyn + L::own;
  unsigned char* s_bq = s_dyn + L::bq;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = static_cast<int>(cl.block_rank());
  const int cidx = static_cast<int>(blockIdx.x) / CS;
  const int r = a.order ? a.order[cidx] : cidx;
  const RepInfo ri = a.reps[r];
  const int n = ri.n_mono;
  // uniform over the cluster (one replica); no CTA has touched another's memory
  if (n == 0 || n > CAP || (ri.flags & REP_PERIODIC_MD)) return;
  const int own = (n - rank + CS - 1) / CS;  // beads rank + CS q, q < own
  int lk = 0;  // log2 of the lanes per bead
  if (KMAX > 1)
    while ((2 << lk) <= KMAX && (own << (lk + 1)) <= NT) ++lk;
  const int sub = static_cast<int>(threadIdx.x) & ((1 << lk) - 1);
  const int q = static_cast<int>(threadIdx.x) >> lk;
  const bool mine = q < own;
  const int i = rank + CS * q;  // this lane's bead (when mine)
  const bool lead = sub == 0;
  const int nl = 1 << lk;  // lanes per bead
  const int b = ri.mono_base;
  const R dt = static_cast<R>(ri.md_dt);
  const R dth = dt * R(0.50);
  const R lambda = static_cast<R>(ri.lambda);
  const R rv2 = static_cast<R>(ri.r_verlet) * static_cast<R>(ri.r_verlet);
  const R lim = (static_cast<R>(ri.r_verlet) - static_cast<R>(ri.r_cut)) * R(0.5);
  const int pot = ri.potential;
  const unsigned long long md_step0 = a.dyn[r].md_step;

  // every CTA: all positions and types; this lane: its bead's state
  if (threadIdx.x == 0) {
    s_far = 0; s_fits = 0;
    s_farp[0] = s_farp[1] = 0;
    s_rebuild[0] = a.force_rebuild; s_rebuild[1] = 0;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += NT) {  // into buffer 0 (substep 0 reads it)
    const R4<R> p = ld4_rw(mpos, b + j);
    s_posr[j] = p.x; s_posr[CAP + j] = p.y; s_posr[2 * CAP + j] = p.z;
    if (kF64) {
      s_posf[j] = static_cast<float>(p.x); s_posf[CAP + j] = static_cast<float>(p.y);
      s_posf[2 * CAP + j] = static_cast<float>(p.z);
    }
    const R4<R> pv = ld4_rw(mver, b + j);
    s_xvf[j] = static_cast<float>(pv.x); s_xvf[CAP + j] = static_cast<float>(pv.y);
    s_xvf[2 * CAP + j] = static_cast<float>(pv.z);
    if (j == 0) {
      s_coref[0] = static_cast<float>(pv.x); s_coref[1] = static_cast<float>(pv.y);
      s_coref[2] = static_cast<float>(pv.z);
    }
    if (!(fabs(p.x) < R(MDC_FAR) && fabs(p.y) < R(MDC_FAR) && fabs(p.z) < R(MDC_FAR))) s_far = 1;
    s_amphi[j] = static_cast<unsigned char>(static_cast<int>(ld4_rw(mvel, b + j).w) & 1);
  }
  // flattened bonds of this CTA's beads (bead slot, partner | anchor << 16)
  bool bonds_fit = false;
  if (threadIdx.x < 32) {
    int carry = 0;
    for (int q0 = 0; q0 < own; q0 += 32) {
      const int qq = q0 + static_cast<int>(threadIdx.x);
      const int ib = b + rank + CS * qq;
      const int cnt = qq < own ? a.bond_start[ib + 1] - a.bond_start[ib] : 0;
      const int inc = md_warp_scan(cnt);
      if (qq < own) s_bstart[qq] = carry + inc - cnt;
      carry += __shfl_sync(0xFFFFFFFFu, inc, 31);
    }
    if (threadIdx.x == 0) s_bstart[own] = carry;
  }
  __syncthreads();
  bonds_fit = s_bstart[own] <= MDC_BCAP;
  if (bonds_fit && static_cast<int>(threadIdx.x) < own) {
    const int ib = rank + CS * static_cast<int>(threadIdx.x);
    int o = s_bstart[threadIdx.x];
    for (int e = a.bond_start[b + ib]; e < a.bond_start[b + ib + 1]; ++e, ++o) {
      const int2 bd = a.bonds[e];
      s_bj[o] = (bd.x - b) | (bd.y != 0 ? 0x10000 : 0);
      s_bq[o] = static_cast<unsigned char>(threadIdx.x);
    }
  }
  // The CTA's Verlet lists flattened into shared memory, bead by bead in list
  // order, from the global lists (written by this CTA and synchronised).
  auto flatten = [&]() {
    if (threadIdx.x < 32) {
      int carry = 0;
      bool bad = false;
      for (int q0 = 0; q0 < own; q0 += 32) {
        const int qq = q0 + static_cast<int>(threadIdx.x);
        int cnt = qq < own ? a.ncount[b + rank + CS * qq] : 0;
        if (cnt < 0 || cnt > a.max_nb) { bad = true; cnt = 0; }
        const int inc = md_warp_scan(cnt);
        if (qq < own) s_lstart[qq] = carry + inc - cnt;
        carry += __shfl_sync(0xFFFFFFFFu, inc, 31);
      }
      bad = __any_sync(0xFFFFFFFFu, bad);
      if (threadIdx.x == 0) {
        s_lstart[own] = carry;
        s_fits = !bad && carry <= MDC_ECAP;
      }
    }
    __syncthreads();
    if (s_fits) {
      const int E = s_lstart[own];
      const size_t stride = static_cast<size_t>(a.n_mono_total);
      for (int k = threadIdx.x; k < E; k += NT) {
        int lo = 0, hi = own - 1;  // the bead slot q with s_lstart[q] <= k < s_lstart[q + 1]
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_lstart[mid] <= k) lo = mid; else hi = mid - 1;
        }
        const int e = k - s_lstart[lo];
        const int* row = a.nlist + static_cast<size_t>(e) * stride;
        s_nb[k] = static_cast<unsigned short>(row[b + rank + CS * lo] - b);
        s_own[k] = static_cast<unsigned char>(lo);
      }
    }
    __syncthreads();
  };
  // x: the position of this lane's bead in the force pass (from shared
  // memory); the bead's dynamic state lives with its kick thread
  R x[3] = {R(0), R(0), R(0)};
  const int kq = static_cast<int>(threadIdx.x);  // kick thread of bead slot kq
  const bool kicker = kq < own;
  const int ik = rank + CS * kq;
  R xk[3] = {R(0), R(0), R(0)}, v[3] = {R(0), R(0), R(0)}, f[3] = {R(0), R(0), R(0)},
    xv[3] = {R(0), R(0), R(0)}, m = R(1);
  // the half-kick increment f / m dt / 2 (Thermostat_None.cpp:22,34), taken
  // once per force evaluation: the second half-kick of a substep and the
  // first of the next use the same force
  R fk[3] = {R(0), R(0), R(0)};
  if (kicker) {
    const R4<R> p = ld4_rw(mpos, b + ik), vv = ld4_rw(mvel, b + ik), ff = ld4_rw(mfrc, b + ik),
                pv = ld4_rw(mver, b + ik);
    xk[0] = p.x; xk[1] = p.y; xk[2] = p.z; m = p.w;
    v[0] = vv.x; v[1] = vv.y; v[2] = vv.z;
    f[0] = ff.x; f[1] = ff.y; f[2] = ff.z;
    xv[0] = pv.x; xv[1] = pv.y; xv[2] = pv.z;
    for (int d = 0; d < 3; ++d) fk[d] = a.andersen ? f[d] * (dth / m) : (f[d] / m) * dth;
  }
  cl.sync();  // every copy loaded before any CTA writes into another's
  if (!a.force_rebuild) flatten();  // (a forced rebuild flattens the new lists)
  int rebuilds = 0;
  double epot = 0.0;
  const int total_steps = a.n_steps > 0 ? a.n_steps : 1;
  for (int step = 0; step < total_steps; ++step) {
    const int cur = step & 1;
    R* const sx = s_posr + cur * 3 * CAP;
    R* const sy = sx + CAP;
    R* const sz = sy + CAP;
    // FP32 positions for the range pre-tests (the state itself in FP32)
    float* const pxf = kF64 ? s_posf + cur * 3 * CAP : reinterpret_cast<float*>(sx);
    float* const pyf = pxf + CAP;
    float* const pzf = pyf + CAP;
    if (a.n_steps > 0 && kicker) {
      // kick + drift (Thermostat_None.cpp:22-27); the force lanes read the
      // new position from shared memory after the barrier
      for (int d = 0; d < 3; ++d) {
        v[d] += fk[d];
        xk[d] += v[d] * dt;
      }
      {
        bool over = false;
        if (!a.core_relative) {  // Box::check_VerletLists (Box.cpp:182-194)
          const R d0 = xk[0] - xv[0], d1 = xk[1] - xv[1], d2 = xk[2] - xv[2];
          over = r_sqrt((d0 * d0 + d1 * d1) + d2 * d2) > lim;
        }
        const bool far = !(fabs(xk[0]) < R(MDC_FAR) && fabs(xk[1]) < R(MDC_FAR) &&
                           fabs(xk[2]) < R(MDC_FAR));
        // this CTA's copy here; the other CTAs' below, by all threads
        sx[ik] = xk[0];
        sy[ik] = xk[1];
        sz[ik] = xk[2];
        if (kF64) {
          pxf[ik] = static_cast<float>(xk[0]);
          pyf[ik] = static_cast<float>(xk[1]);
          pzf[ik] = static_cast<float>(xk[2]);
        }
        if (over || far)
          for (int c = 0; c < CS; ++c) {
            if (over) *cl.map_shared_rank(&s_rebuild[cur], c) = 1;
            if (far) *cl.map_shared_rank(&s_farp[cur], c) = 1;
          }
      }
    }
    if (a.n_steps > 0) {
      // Positions into the other CTAs' copies: one (bead, CTA) pair per
      // thread, from this CTA's copy; one address mapping per pair (the
      // buffers lie at fixed offsets in the dynamic shared memory).
      __syncthreads();
      const size_t ox = reinterpret_cast<const unsigned char*>(sx) - s_dyn;
      const size_t of = reinterpret_cast<const unsigned char*>(pxf) - s_dyn;
      for (int t = threadIdx.x; t < own * (CS - 1); t += NT) {
        const int bq = t / (CS - 1);
        const int c0 = t - bq * (CS - 1);
        const int c = c0 + (c0 >= rank ? 1 : 0);
        const int ib = rank + CS * bq;
        unsigned char* base = cl.map_shared_rank(s_dyn, c);
        R* rx = reinterpret_cast<R*>(base + ox);
        rx[ib] = sx[ib];
        rx[CAP + ib] = sy[ib];
        rx[2 * CAP + ib] = sz[ib];
        if (kF64) {
          float* fx = reinterpret_cast<float*>(base + of);
          fx[ib] = pxf[ib];
          fx[CAP + ib] = pyf[ib];
          fx[2 * CAP + ib] = pzf[ib];
        }
      }
    }
    cl.sync();  // positions and flags of this substep complete in every CTA
    if (mine) { x[0] = sx[i]; x[1] = sy[i]; x[2] = sz[i]; }
    const bool far_now = s_far || s_farp[cur];
    bool over_here = s_rebuild[cur] != 0;
    if (a.core_relative && a.n_steps > 0) {
      // Displacements relative to the core's (see k_md_substeps), decided by
      // every CTA for every bead from the same FP32 positions, so all CTAs
      // agree without a second cluster barrier. FP32 states compare with
      // lim^2 as k_md_substeps; FP64 states with (lim - 2e-3)^2, which
      // covers the FP32 rounding of coordinates below MDC_FAR (a rebuild a
      // little early keeps the lists valid), and rebuild at every substep
      // once a coordinate reaches MDC_FAR.
      const float limf = static_cast<float>(lim);
      const float limm = limf > 2e-3f ? limf - 2e-3f : 0.0f;
      const float thr = kF64 ? limm * limm : limf * limf;
      if (kF64 && far_now) {
        over_here = true;
      } else {
        const float c0 = pxf[0] - s_coref[0], c1 = pyf[0] - s_coref[1], c2 = pzf[0] - s_coref[2];
        for (int j = threadIdx.x; j < n; j += NT) {
          const float d0 = pxf[j] - s_xvf[j] - c0, d1 = pyf[j] - s_xvf[CAP + j] - c1,
                      d2 = pzf[j] - s_xvf[2 * CAP + j] - c2;
          if ((d0 * d0 + d1 * d1) + d2 * d2 > thr) over_here = true;
        }
      }
    }
    const int rebuild = __syncthreads_or(over_here);  // the same in every CTA
    if (threadIdx.x == 0) {  // set again by the pushes of substep step + 2
      s_rebuild[cur] = 0;
      if (far_now) s_far = 1;
    }
    if (rebuild) {
      ++rebuilds;
      const R inv_rv = R(1) / static_cast<R>(ri.r_verlet);
      for (int j = threadIdx.x; j < n; j += NT) {
        const int cx = static_cast<int>(floor(sx[j] * inv_rv));
        const int cy = static_cast<int>(floor(sy[j] * inv_rv));
        const int cz = static_cast<int>(floor(sz[j] * inv_rv));
        s_ckey[j] = md_cell_key(cx, cy, cz);
        s_next[j] = md_bucket(cx, cy, cz);
      }
      __syncthreads();
      md_bucket_sort<NT>(n, s_next, s_head, s_sorted);
      // Lists: the lanes of a bead split its 27 cells (cell t to lane t mod
      // lanes), count their members, then write them at the offsets the
      // counts give, so a list holds lane 0's cells, then lane 1's, and so
      // on. Membership is d^2 <= r_v^2 in the state's precision; FP64 states
      // decide it in FP32 outside a band of 2^-7 around r_v^2 (FP32 rounding
      // of coordinates below MDC_FAR moves d^2 by far less) and in FP64
      // inside it.
      const bool fast = kF64 && !far_now;
      const float rv2_lo = static_cast<float>(rv2) * (1.0f - 0.0078125f);
      const float rv2_hi = static_cast<float>(rv2) * (1.0f + 0.0078125f);
      int ccx = 0, ccy = 0, ccz = 0;
      float xf0 = 0.f, xf1 = 0.f, xf2 = 0.f;
      if (mine) {
        ccx = static_cast<int>(floor(x[0] * inv_rv));
        ccy = static_cast<int>(floor(x[1] * inv_rv));
        ccz = static_cast<int>(floor(x[2] * inv_rv));
        xf0 = pxf[i]; xf1 = pyf[i]; xf2 = pzf[i];
      }
      // members of this lane's cells: counted (pos < 0) or written from pos
      // emit(j) for every member of this lane's cells, in order; members
      // are examined four at a time, their loads in flight together
      auto walk = [&](auto&& emit) {
        for (int t = sub; t < 27; t += nl) {
          const int tx = ccx + t % 3 - 1, ty = ccy + (t / 3) % 3 - 1, tz = ccz + t / 9 - 1;
          const int want = md_cell_key(tx, ty, tz);
          const int bk = md_bucket(tx, ty, tz);
          const int kend = s_head[bk + 1];
          for (int kk = s_head[bk]; kk < kend; kk += 4) {
            int jj[4], kc[4];
            float e0[4], e1[4], e2[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) jj[u] = kk + u < kend ? s_sorted[kk + u] : -1;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int j = jj[u] < 0 ? 0 : jj[u];
              kc[u] = s_ckey[j];
              e0[u] = pxf[j] - xf0;
              e1[u] = pyf[j] - xf1;
              e2[u] = pzf[j] - xf2;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int j = jj[u];
              if (j < 0 || j == i || kc[u] != want) continue;
              bool in;
              const float r2f = fmaf(e0[u], e0[u], fmaf(e1[u], e1[u], e2[u] * e2[u]));
              if (fast && r2f < rv2_lo) {
                in = true;
              } else if (fast && r2f > rv2_hi) {
                in = false;
              } else {
                const R d0 = sx[j] - x[0], d1 = sy[j] - x[1], d2 = sz[j] - x[2];
                in = (d0 * d0 + d1 * d1) + d2 * d2 <= rv2;
              }
              if (in) emit(j);
            }
          }
        }
      };
      // Pass 1 counts the members and keeps the first MDC_SCRATCH of each
      // lane in scratch (the candidate buffer, idle here; slot e of thread t
      // at e NT + t); the lists are then copied from there, or, if any lane
      // found more, written by a second walk.
      constexpr int MDC_SCRATCH = MDC_ECAP / NT;
      int mc = 0;
      if (mine)
        walk([&](int j) {
          if (mc < MDC_SCRATCH) s_cand[mc * NT + threadIdx.x] = j;
          ++mc;
        });
      int inc = mc;  // the bead's lanes are adjacent: segments of nl lanes
      for (int o = 1; o < nl; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, inc, o, nl);
        if (sub >= o) inc += t;
      }
      const int total = __shfl_sync(0xFFFFFFFFu, inc, nl - 1, nl);
      if (mine && lead) {
        int cnt = total;
        if (cnt > a.max_nb) {
          raise_error(a.err, ERR_NEIGHBOR_OVF, static_cast<uint32_t>(b + i),
                      static_cast<uint32_t>(cnt));
          cnt = a.max_nb;
        }
        a.ncount[b + i] = cnt;
        s_cstart[q] = cnt;
      }
      const int spill = __syncthreads_or(mc > MDC_SCRATCH);
      if (threadIdx.x < 32) {  // list starts of the CTA's beads
        int carry = 0;
        for (int q0 = 0; q0 < own; q0 += 32) {
          const int qq = q0 + static_cast<int>(threadIdx.x);
          const int cnt = qq < own ? s_cstart[qq] : 0;
          const int ci = md_warp_scan(cnt);
          if (qq < own) s_lstart[qq] = carry + ci - cnt;
          carry += __shfl_sync(0xFFFFFFFFu, ci, 31);
        }
        if (threadIdx.x == 0) {
          s_lstart[own] = carry;
          s_fits = carry <= MDC_ECAP;
        }
      }
      __syncthreads();
      if (mine) {
        int k = inc - mc;  // this lane's first list position
        auto put = [&](int j) {
          if (k < a.max_nb) {
            a.nlist[static_cast<size_t>(k) * a.n_mono_total + b + i] = b + j;
            if (s_fits) {
              s_nb[s_lstart[q] + k] = static_cast<unsigned short>(j);
              s_own[s_lstart[q] + k] = static_cast<unsigned char>(q);
            }
          }
          ++k;
        };
        if (!spill) {
          for (int e = 0; e < mc; ++e) put(s_cand[e * NT + threadIdx.x]);
        } else {
          walk(put);
        }
      }
      if (kicker) { xv[0] = xk[0]; xv[1] = xk[1]; xv[2] = xk[2]; }
      for (int j = threadIdx.x; j < n; j += NT) {
        s_xvf[j] = pxf[j]; s_xvf[CAP + j] = pyf[j]; s_xvf[2 * CAP + j] = pzf[j];
      }
      if (threadIdx.x == 0) { s_coref[0] = pxf[0]; s_coref[1] = pyf[0]; s_coref[2] = pzf[0]; }
      __syncthreads();  // lists written before the lanes of a bead read them
    }
    const bool want_epot = a.calc_epot && (step == total_steps - 1);
    // forces (Box.cpp:243-286)
    if (bonds_fit && s_fits && !far_now) {
      // 1. candidates, by warp over contiguous runs of the flattened lists
      const int E = s_lstart[own];
      const int w = static_cast<int>(threadIdx.x >> 5), lane = static_cast<int>(threadIdx.x & 31u);
      const int per = (E + NW - 1) / NW;
      const int k0 = w * per, k1 = min(E, k0 + per);
      const float widen = 1.0f + 0.0078125f;
      const float cut_aa = (pot == POT_REF4824 ? 1.0594631f : 1.2599211f) * widen;
      const float cut_bb = (pot == POT_REF4824 ? 2.25f : 6.25f) * widen;
      int nw = 0;
      for (int kb = k0, rd = 0; kb < k1; kb += 32, ++rd) {
        const int k = kb + lane;
        bool cand = false;
        int pk = 0;
        if (k < k1) {
          const int qk = s_own[k];
          const int j = s_nb[k], ii = rank + CS * qk;
          const float d0 = pxf[j] - pxf[ii], d1 = pyf[j] - pyf[ii], d2 = pzf[j] - pzf[ii];
          const float r2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
          cand = r2 < ((s_amphi[ii] != 0 && s_amphi[j] != 0) ? cut_bb : cut_aa);
          pk = (qk << 10) | j;
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, cand);
        if (cand) s_cand[k0 + nw + __popc(m & ((1u << lane) - 1u))] = pk;
        if (lane == 0) {
          s_rpre[rd][w] = nw;
          s_rmask[rd][w] = m;
        }
        nw += __popc(m);
      }
      if (lane == 0) s_wcnt[w] = nw;
      __syncthreads();
      // candidate offsets by warp, in every thread (eight counts)
      int woff[NW + 1];
      woff[0] = 0;
#pragma unroll
      for (int u = 0; u < NW; ++u) woff[u + 1] = woff[u] + s_wcnt[u];
      const int C = woff[NW];
      if (threadIdx.x <= NW) {  // for the bead ranges below (read after a barrier)
#pragma unroll
        for (int u = 0; u <= NW; ++u)
          if (u == static_cast<int>(threadIdx.x)) s_woff[u] = woff[u];
      }
      // candidates before list position kq: those of the earlier warps, of
      // the earlier rounds of its warp, and of the earlier lanes of its round
      auto cand_before = [&](int kq) -> int {
        if (kq >= E) return C;
        const int wq = kq / per, o = kq - wq * per;
        const unsigned below = (1u << (o & 31)) - 1u;
        return s_woff[wq] + s_rpre[o >> 5][wq] + __popc(s_rmask[o >> 5][wq] & below);
      };
      R F0 = R(0), F1 = R(0), F2 = R(0);
      for (int c0 = 0; c0 == 0 || c0 < C; c0 += MDC_CCAP) {
        const int c1 = min(C, c0 + MDC_CCAP);
        // 2. FP64 pair forces of the candidates, then the bonds (first batch)
        for (int c = c0 + static_cast<int>(threadIdx.x); c < c1; c += NT) {
          int wc = 0, wb = 0;  // the warp whose region holds candidate c
#pragma unroll
          for (int u = 1; u < NW; ++u)
            if (woff[u] <= c) { wc = u; wb = woff[u]; }
          const int pk = s_cand[wc * per + (c - wb)];
          const int qk = pk >> 10, j = pk & 1023, ii = rank + CS * qk;
          const R d0 = sx[j] - sx[ii], d1 = sy[j] - sy[ii], d2 = sz[j] - sz[ii];
          const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
          const bool bb = s_amphi[ii] != 0 && s_amphi[j] != 0;
          const R fa = pair_force<R>(pot, bb, r2, lambda);
          R* o = s_pf + 3 * (c - c0);
          o[0] = d0 * fa;
          o[1] = d1 * fa;
          o[2] = d2 * fa;
          if (want_epot) epot += md_pair_epot<R>(pot, bb, r2, lambda);
        }
        if (c0 == 0) {
          for (int e = threadIdx.x; e < s_bstart[own]; e += NT) {
            const int ii = rank + CS * s_bq[e], j = s_bj[e] & 0xFFFF;
            const bool anch = (s_bj[e] >> 16) != 0;
            const R d0 = sx[j] - sx[ii], d1 = sy[j] - sy[ii], d2 = sz[j] - sz[ii];
            const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
            R r2f = r2;
            if (pot == POT_REF4824) {
              if (r2 >= (anch ? R(20.25) : R(2.25)))
                raise_error(a.err, ERR_FENE, static_cast<uint32_t>(b + ii),
                            static_cast<uint32_t>(b + j));
            } else {
              const R cap = (anch ? R(20.25) : R(2.25)) * R(0.98);
              if (r2f > cap) r2f = cap;
            }
            const R fa = fene_force<R>(anch, r2f);
            R* o = s_bf + 3 * e;
            o[0] = d0 * fa;
            o[1] = d1 * fa;
            o[2] = d2 * fa;
            if (want_epot) epot += md_fene_epot<R>(anch, r2f);
          }
        }
        __syncthreads();
        // 3. each bead's lanes: lane sub takes the bead's candidates
        // cs + sub, cs + sub + lanes, ... (cs its first)
        if (mine) {
          const int cs = cand_before(s_lstart[q]), e1 = min(cand_before(s_lstart[q + 1]), c1);
          const int st = max(cs, c0);
          for (int c = st + (((sub - (st - cs)) % nl) + nl) % nl; c < e1; c += nl) {
            const R* o = s_pf + 3 * (c - c0);
            F0 -= o[0];
            F1 -= o[1];
            F2 -= o[2];
          }
        }
        __syncthreads();  // read before the next batch rewrites the buffer
      }
      if (mine) {  // then its bonds, the same way
        for (int e = s_bstart[q] + sub; e < s_bstart[q + 1]; e += nl) {
          F0 -= s_bf[3 * e];
          F1 -= s_bf[3 * e + 1];
          F2 -= s_bf[3 * e + 2];
        }
      }
      for (int o = 1; o < nl; o <<= 1) {  // whole warps take part
        F0 += __shfl_xor_sync(0xFFFFFFFFu, F0, o);
        F1 += __shfl_xor_sync(0xFFFFFFFFu, F1, o);
        F2 += __shfl_xor_sync(0xFFFFFFFFu, F2, o);
      }
      if (mine && lead) {
        s_f[3 * q] = F0;
        s_f[3 * q + 1] = F1;
        s_f[3 * q + 2] = F2;
      }
    } else {
    R F[3] = {R(0), R(0), R(0)};
    if (mine)
      md_bead_forces_lists<R>(a, b, i, sub, lk, lead, sx, sy, sz, s_amphi, pot, lambda, want_epot,
                              F, &epot);
    R F0 = F[0], F1 = F[1], F2 = F[2];
    for (int o = 1; KMAX > 1 && o < (1 << lk); o <<= 1) {  // whole warps take part
      F0 += __shfl_xor_sync(0xFFFFFFFFu, F0, o);
      F1 += __shfl_xor_sync(0xFFFFFFFFu, F1, o);
      F2 += __shfl_xor_sync(0xFFFFFFFFu, F2, o);
    }
    if (mine && lead) {
      s_f[3 * q] = F0;
      s_f[3 * q + 1] = F1;
      s_f[3 * q + 2] = F2;
    }
    }
    __syncthreads();  // the forces reach the kick threads
    if (kicker) {
      f[0] = s_f[3 * kq];
      f[1] = s_f[3 * kq + 1];
      f[2] = s_f[3 * kq + 2];
      for (int d = 0; d < 3; ++d) fk[d] = a.andersen ? f[d] * (dth / m) : (f[d] / m) * dth;
      if (a.n_steps > 0) {
        for (int d = 0; d < 3; ++d)  // second half-kick
          v[d] += fk[d];
        if (a.andersen) md_andersen_reset<R>(a, ri, r, step, ik, md_step0, m, v);
      }
    }
  }
  if (kicker) {
    R4<R> p = ld4_rw(mpos, b + ik);
    p.x = xk[0]; p.y = xk[1]; p.z = xk[2];
    st4(mpos, b + ik, p);
    R4<R> vv = ld4_rw(mvel, b + ik);
    vv.x = v[0]; vv.y = v[1]; vv.z = v[2];
    st4(mvel, b + ik, vv);
    st4(mfrc, b + ik, R4<R>{f[0], f[1], f[2], R(0)});
    st4(mver, b + ik, R4<R>{xv[0], xv[1], xv[2], R(0)});
  }
  if (a.calc_epot) {
    for (int o = 16; o > 0; o >>= 1) epot += __shfl_down_sync(0xFFFFFFFFu, epot, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = epot;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < NT / 32; ++w) s += s_red[w];
      cl.map_shared_rank(s_epot, 0)[rank] = s;
    }
    cl.sync();  // the partial sums are in CTA 0 (and nobody reads another CTA after this)
    if (rank == 0 && threadIdx.x == 0) {
      double s = 0.0;
      for (int c = 0; c < CS; ++c) s += s_epot[c];
      a.dyn[r].epot = s;
    }
  }
  if (rank == 0 && threadIdx.x == 0) {
    a.dyn[r].verlet_rebuilds += rebuilds;
    if (a.n_steps > 0) a.dyn[r].md_step = md_step0 + static_cast<unsigned long long>(a.n_steps);
  }
}

}  // namespace smpc
