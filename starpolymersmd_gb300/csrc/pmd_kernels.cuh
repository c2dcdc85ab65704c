// Periodic molecular dynamics of many stars in one sheared box (semi-dilute
// solutions): the velocity-Verlet substep, FENE bonds and pair forces of
// md_kernels.cuh (Thermostat_None::propagate, Thermostat_None.cpp:21-38;
// Potentials.h:14-120), with every pair distance taken as the Lees-Edwards
// minimum image at the substep's delrx (the operations of
// MPC::relative_position, MPC.cpp:456-465), beads kept in the primary box by
// the shift and v_x jump of MPC::LEBC (MPC.cpp:421-429), and Verlet lists
// built on a periodic cell grid. The reference integrates one star without
// periodic images (Box.cpp:105-180); several interacting stars in one box
// need this form.
//
// A call of n substeps (k = 1..n) is 2n + 1 launches, plus a copy when n is
// even:
//   k_pmd_drift   substep 1: half kick and drift, Lees-Edwards wrap, peculiar
//                 displacement, binning into the grid of substep 1, rebuild
//                 request; block 0 records the substep's delrx
//   k_pmd_nlist   (rebuild only, else it returns at once) one warp per bead: the lanes
//                 test the beads of the 27 neighbour cells (across a y face
//                 the neighbour rows are looked up at x -/+ delrx) and the
//                 list is written in bead-index order, so the force sums do
//                 not depend on the order the binning atomics filled the
//                 cells in. Lists are rows of max_nb entries per bead.
//   k_pmd_forces  LANES lanes per bead split its Verlet list, a butterfly sums
//                 them; second half kick; then, for k < n, substep k+1's half
//                 kick, drift, wrap and binning, writing the positions into
//                 the other of two position buffers (other beads still read
//                 substep k's); the last block to finish records the new
//                 lists' delrx, clears the request, sums the potential
//                 energy of the blocks in a fixed order, and records delrx
//                 and the rebuild threshold of substep k + 2 (the drift
//                 kernel's last block those of substep 2)
// Substep k's positions live in buffer (k - 1) & 1 (0 = the monomer array),
// its grid, rebuild request and delrx in slots k & 1. The set-up call (n = 0)
// wraps, bins and builds lists and forces at the current positions.
//
// Rebuild criterion. The Verlet-reference array of a periodic box holds each
// bead's peculiar displacement since the last build, u = sum (v - shear y e_x)
// dt with y the bead's height at the start of the drift (continuous across a
// y face, where y and v_x jump together). Lees-Edwards images move with the
// affine flow, so over a time t the minimum-image separation of any two beads
// changes by u_j - u_i plus shear * t times their image-frame height
// difference, which is at most r_verlet + skin for every pair that can come
// within r_cut. A pair outside the lists then stays outside r_cut while
//   2 max|u| + shear t (r_verlet + skin) + |delrx drift| <= skin,
// where the delrx drift is the part of the change of delrx since the build
// that the flow does not explain (zero in the physical delrx mode, up to
// round-off; the reference mode advances delrx faster than the flow). Beads
// carried by the shear flow therefore trigger no rebuilds.
#pragma once
#include <stdint.h>

#include <type_traits>

#include "md_kernels.cuh"
#include "observables.cuh"

namespace smpc {

constexpr int PMD_CELL_CAP = 128;  // beads per grid cell
constexpr int PMD_NT = 256;        // threads per block of every periodic-MD kernel
constexpr int PMD_NL_CAP = 256;    // Verlet-list entries one warp of k_pmd_nlist collects

// Lanes per bead in k_pmd_forces: FP64 keeps one (the oracle's order of the
// sums); FP32 splits each list over eight by default, or over 4 or 16 (the
// launch-shape variants of the periodic MD, pmd_variant_*).
constexpr int PMD_MAX_LANES = 16;
template <typename R>
constexpr int pmd_force_lanes() {
  return std::is_same<R, float>::value ? 8 : 1;
}

inline int pmd_force_block_count(int n_beads, int lanes) {
  return (n_beads * lanes + PMD_NT - 1) / PMD_NT;
}

struct PmdArgs {
  int rep;
  int base;            // first global monomer of the box
  int n;               // beads
  int nc[3];           // grid cells per axis (>= 3, side >= r_verlet)
  int ncell;
  int n_blocks;        // blocks of the one-thread-per-bead launches
  uint32_t* cnt[2];    // beads per grid cell, grids of even / odd substeps
  int* items[2];       // ncell x PMD_CELL_CAP bead indices (box-local)
  int* flag;           // [0], [1] rebuild requested (even / odd substep),
                       // [2] blocks done, [3] substeps since the last build
  double* delrx_build; // delrx of the current lists
  double* dl_slot;     // substep k: delrx at [k & 1], rebuild threshold at [2 + (k & 1)]
  double* epot_part;   // per block of k_pmd_forces
  int* nlist;          // [n][max_nb] global indices of each bead's Verlet list
  int* ncount;         // per global monomer
  const uint8_t* amphi;  // per global monomer: 1 = solvophobic
  int n_mono_total;
  int max_nb;
  const int* bond_start;
  const int2* bonds;
  ErrorState* err;
  int andersen;        // Andersen stochastic thermostat (MPC-off runs), md_kernels.cuh
  double andersen_nu;
};

// delrx one MD step later: one iteration of k_cycle_begin's loop
// (MPC.cpp:117-118), so substep k of a call sees k of them
__device__ __forceinline__ double pmd_advance(const RepInfo& ri, double d, double adv_scale) {
  const double Lx = static_cast<double>(ri.L[0]);
  const double adv_dt = __dmul_rn(ri.h, adv_scale);
  d = __dadd_rn(d, __dmul_rn(__dmul_rn(ri.shear, static_cast<double>(ri.L[1])), adv_dt));
  return __dsub_rn(d, __dmul_rn(Lx, round(__ddiv_rn(d, Lx))));
}

// q / L: a division in FP64 (the reference's operation), the reciprocal
// product in FP32 (only which of two equivalent images is taken differs)
__device__ __forceinline__ double pmd_ratio(double q, double L, double) { return q / L; }
__device__ __forceinline__ float pmd_ratio(float q, float, float invL) { return q * invL; }

template <typename R>
struct PmdBox {
  R L[3];
  R inv[3];
  R delrx;
};

template <typename R>
__device__ __forceinline__ PmdBox<R> pmd_box(const RepInfo& ri, double dl) {
  PmdBox<R> b;
  for (int d = 0; d < 3; ++d) {
    b.L[d] = static_cast<R>(ri.L[d]);
    b.inv[d] = R(1) / b.L[d];
  }
  b.delrx = static_cast<R>(dl);
  return b;
}

// Lees-Edwards minimum image of d = x_j - x_i: FP64 with the operations of
// MPC::relative_position (MPC.cpp:456-465); FP32 with one wrap of x after the
// shift and rint (the same image, away from exact half-box separations,
// which no Verlet pair has)
__device__ __forceinline__ void pmd_min_image(double& dx, double& dy, double& dz,
                                              const PmdBox<double>& b) {
  const double cy = round(dy / b.L[1]);
  dx -= b.L[0] * round(dx / b.L[0]);
  dx -= cy * b.delrx;
  dx -= b.L[0] * round(dx / b.L[0]);
  dy -= b.L[1] * cy;
  dz -= b.L[2] * round(dz / b.L[2]);
}
__device__ __forceinline__ void pmd_min_image(float& dx, float& dy, float& dz,
                                              const PmdBox<float>& b) {
  const float cy = rintf(dy * b.inv[1]);
  dx -= cy * b.delrx;
  dx -= b.L[0] * rintf(dx * b.inv[0]);
  dy -= b.L[1] * cy;
  dz -= b.L[2] * rintf(dz * b.inv[2]);
}

template <typename R>
__device__ __forceinline__ int pmd_cell_axis(R x, R L, int nc) {
  const int c = static_cast<int>(r_floor((x + R(0.5) * L) * (static_cast<R>(nc) / L)));
  return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

template <typename R>
__device__ __forceinline__ int pmd_cell(const PmdArgs& a, const PmdBox<R>& b, const R4<R>& x) {
  return pmd_cell_axis(x.x, b.L[0], a.nc[0]) +
         a.nc[0] * (pmd_cell_axis(x.y, b.L[1], a.nc[1]) +
                    a.nc[1] * pmd_cell_axis(x.z, b.L[2], a.nc[2]));
}

// Rebuild threshold of a substep whose drift ends `tb` after the last build
// at delrx `db`, at delrx `dl` (criterion in the header comment).
template <typename R>
__device__ __forceinline__ R pmd_threshold(const RepInfo& ri, double dl, double db, R tb) {
  const R Lx = static_cast<R>(ri.L[0]);
  const R shear = static_cast<R>(ri.shear);
  const R skin = static_cast<R>(ri.r_verlet) - static_cast<R>(ri.r_cut);
  R ddl = static_cast<R>(dl - db) - shear * static_cast<R>(ri.L[1]) * tb;
  ddl -= Lx * r_round(ddl / Lx);
  return R(0.5) * (skin - r_fabs(shear) * tb * (static_cast<R>(ri.r_verlet) + skin) - r_fabs(ddl));
}

// Records delrx and the rebuild threshold of the substep after substep k
// (slot s = k & 1), once k's rebuild request is final: its lists will be k's
// if k rebuilds them, else the older ones.
template <typename R>
__device__ __forceinline__ void pmd_next_constants(const PmdArgs& a, const RepInfo& ri, int s,
                                                   double adv_scale) {
  const double dl = a.dl_slot[s];
  const int rebuilt = a.flag[s];
  const double dl1 = pmd_advance(ri, dl, adv_scale);
  const double db = rebuilt ? dl : *a.delrx_build;
  const int since = rebuilt ? 0 : a.flag[3] + 1;
  a.dl_slot[s ^ 1] = dl1;
  a.dl_slot[2 + (s ^ 1)] = static_cast<double>(
      pmd_threshold<R>(ri, dl1, db, static_cast<R>(since + 1) * static_cast<R>(ri.md_dt)));
}

// True in one thread of the last block of the grid to get here; the blocks
// count themselves in flag[2], which that thread resets (no block waits).
__device__ __forceinline__ bool pmd_last_block(const PmdArgs& a) {
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(reinterpret_cast<unsigned*>(a.flag + 2), 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return false;
  __threadfence();
  a.flag[2] = 0;
  return true;
}

// One bead's half kick (with the force f), drift, Lees-Edwards wrap and
// peculiar displacement (Thermostat_None.cpp:22-27, MPC.cpp:421-429).
template <typename R>
__device__ __forceinline__ R pmd_kick(R f, R m, R dth, int andersen) {
  // Thermostat_None.cpp:24; Andersen_stochastic.cpp:33 groups it as f (dt/2 / m)
  return andersen ? f * (dth / m) : (f / m) * dth;
}

template <typename R>
__device__ __forceinline__ void pmd_drift_bead(const RepInfo& ri, const PmdBox<R>& b, R4<R>& x,
                                               R4<R>& v, R4<R>& u, R f0, R f1, R f2,
                                               int andersen) {
  const R dt = static_cast<R>(ri.md_dt), dth = dt * R(0.50);
  const R y0 = x.y;
  v.x += pmd_kick(f0, x.w, dth, andersen);
  x.x += v.x * dt;
  u.x += (v.x - static_cast<R>(ri.shear) * y0) * dt;
  v.y += pmd_kick(f1, x.w, dth, andersen);
  x.y += v.y * dt;
  u.y += v.y * dt;
  v.z += pmd_kick(f2, x.w, dth, andersen);
  x.z += v.z * dt;
  u.z += v.z * dt;
}

template <typename R>
__device__ __forceinline__ void pmd_wrap(const RepInfo& ri, const PmdBox<R>& b, R4<R>& x,
                                         R4<R>& v) {
  const R cy = r_round(pmd_ratio(x.y, b.L[1], b.inv[1]));
  x.x -= b.L[0] * r_round(pmd_ratio(x.x, b.L[0], b.inv[0]));
  x.x -= cy * b.delrx;
  x.x -= b.L[0] * r_round(pmd_ratio(x.x, b.L[0], b.inv[0]));
  x.y -= b.L[1] * cy;
  x.z -= b.L[2] * r_round(pmd_ratio(x.z, b.L[2], b.inv[2]));
  v.x -= cy * static_cast<R>(ri.shear) * b.L[1];
}

// bead i (box-local) into grid s
template <typename R>
__device__ __forceinline__ void pmd_bin(const PmdArgs& a, int s, const PmdBox<R>& b,
                                        const R4<R>& x, int i) {
  const int c = pmd_cell(a, b, x);
  const uint32_t k = atomicAdd(a.cnt[s] + c, 1u);
  if (k < static_cast<uint32_t>(PMD_CELL_CAP))
    a.items[s][static_cast<size_t>(c) * PMD_CELL_CAP + k] = i;
  else
    raise_error(a.err, ERR_NEIGHBOR_OVF, static_cast<uint32_t>(a.base + i), k);
}

// Programmatic dependent launch: the substep kernels after the first are
// launched with cudaLaunchAttributeProgrammaticStreamSerialization, so their
// blocks are scheduled while the previous kernel drains; each waits here,
// before its first read, until that kernel has completed and its writes are
// visible (griddepcontrol.wait; it returns at once for an ordinary launch).
__device__ __forceinline__ void pmd_wait_previous() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Substep 1 of a call (adv_k = 1, drift = 1) or the set-up (adv_k = 0,
// drift = 0: wrap what the caller placed outside, request the first build).
template <typename R>
__global__ void __launch_bounds__(PMD_NT)
    k_pmd_drift(PmdArgs a, const RepInfo* reps, const RepDyn* dyn, R* mpos, R* mvel,
                const R* mfrc, R* mdisp, int adv_k, double adv_scale, int drift) {
  const RepInfo& ri = reps[a.rep];
  __shared__ double s_dl;
  __shared__ R s_thr;
  if (threadIdx.x == 0) {
    const double base = dyn[a.rep].delrx;
    const double dl = adv_k == 0 ? base : pmd_advance(ri, base, adv_scale);
    if (blockIdx.x == 0) a.dl_slot[adv_k & 1] = dl;
    s_dl = dl;
    s_thr = pmd_threshold<R>(ri, dl, *a.delrx_build,
                             static_cast<R>(a.flag[3] + 1) * static_cast<R>(ri.md_dt));
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) {
    const PmdBox<R> b = pmd_box<R>(ri, s_dl);
    const size_t g = static_cast<size_t>(a.base) + i;
    R4<R> x = ld4_rw(mpos, g), v = ld4_rw(mvel, g), u = ld4_rw(mdisp, g);
    if (drift) {
      const R4<R> f = ld4_rw(mfrc, g);
      pmd_drift_bead(ri, b, x, v, u, f.x, f.y, f.z, a.andersen);
    }
    pmd_wrap(ri, b, x, v);
    st4(mpos, g, x);
    st4(mvel, g, v);
    pmd_bin(a, adv_k & 1, b, x, i);
    if (!drift) {
      if (i == 0) a.flag[0] = 1;
    } else {
      st4(mdisp, g, u);
      const R thr = s_thr;
      if (thr <= R(0) || (u.x * u.x + u.y * u.y) + u.z * u.z > thr * thr) a.flag[adv_k & 1] = 1;
    }
  }
  // this substep's request is final: the next substep's constants
  if (pmd_last_block(a)) pmd_next_constants<R>(a, ri, adv_k & 1, adv_scale);
}

// Verlet list of bead i (box-local) by the 32 lanes of one warp; buf holds
// PMD_NL_CAP entries.
template <typename R>
__device__ __forceinline__ void pmd_list_bead(const PmdArgs& a, int s, const PmdBox<R>& b, R rv2,
                                              const R* pos, R* mdisp, int i, int lane, int* buf) {
  constexpr unsigned FULL = 0xFFFFFFFFu;
  const size_t g = static_cast<size_t>(a.base) + i;
  const R4<R> x = ld4_rw(pos, g);
  const int nx = a.nc[0], ny = a.nc[1], nz = a.nc[2];
  const uint32_t* cnt = a.cnt[s];
  const int* items = a.items[s];
  // lanes 0..26: one neighbour cell each (row-major over dz, dy, dx)
  int c_l = 0, m_l = 0;
  if (lane < 27) {
    const int oz = lane / 9 - 1, oy = (lane / 3) % 3 - 1, ox = lane % 3 - 1;
    const int zz = (pmd_cell_axis(x.z, b.L[2], nz) + oz + nz) % nz;
    const int yr = pmd_cell_axis(x.y, b.L[1], ny) + oy;
    const int yy = (yr + ny) % ny;
    // the row beyond a y face is the image shifted by delrx along x
    R xc = x.x;
    if (yr >= ny) xc -= b.delrx;
    if (yr < 0) xc += b.delrx;
    xc -= b.L[0] * r_round(pmd_ratio(xc, b.L[0], b.inv[0]));
    const int cx = pmd_cell_axis(xc, b.L[0], nx);
    c_l = (cx + ox + nx) % nx + nx * (yy + ny * zz);
    m_l = min(static_cast<int>(cnt[c_l]), PMD_CELL_CAP);
  }
  int incl = m_l;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int excl = incl - m_l;
  const int total = __shfl_sync(FULL, incl, 31);
  // the candidates of all 27 cells, 32 at a time: lane k takes candidate k0 + k
  int n_acc = 0;
  for (int k0 = 0; k0 < total; k0 += 32) {
    const int k = k0 + lane;
    int L = 0;  // the cell lane whose range [excl, incl) holds k
    for (int st = 16; st > 0; st >>= 1) {
      const int e = __shfl_sync(FULL, excl, L + st);
      if (L + st < 27 && e <= k) L += st;
    }
    const int cell = __shfl_sync(FULL, c_l, L);
    const int q = k - __shfl_sync(FULL, excl, L);
    bool ok = false;
    int j = -1;
    if (k < total) {
      j = items[static_cast<size_t>(cell) * PMD_CELL_CAP + q];
      if (j != i) {
        const R4<R> y = ld4_rw(pos, static_cast<size_t>(a.base) + j);
        R d0 = y.x - x.x, d1 = y.y - x.y, d2 = y.z - x.z;
        pmd_min_image(d0, d1, d2, b);
        ok = (d0 * d0 + d1 * d1) + d2 * d2 <= rv2;
      }
    }
    const unsigned ball = __ballot_sync(FULL, ok);
    const int at = n_acc + __popc(ball & ((1u << lane) - 1u));
    if (ok && at < PMD_NL_CAP) buf[at] = j;
    n_acc += __popc(ball);
  }
  __syncwarp();
  const int cap = min(a.max_nb, PMD_NL_CAP);
  if (n_acc > cap) {
    if (lane == 0)
      raise_error(a.err, ERR_NEIGHBOR_OVF, static_cast<uint32_t>(g), static_cast<uint32_t>(n_acc));
    n_acc = cap;
  }
  // entry e goes to the place of its rank among the collected indices
  int* row = a.nlist + static_cast<size_t>(i) * a.max_nb;
  for (int e = lane; e < n_acc; e += 32) {
    const int je = buf[e];
    int r = 0;
    for (int f = 0; f < n_acc; ++f) r += buf[f] < je ? 1 : 0;
    row[r] = a.base + je;
  }
  if (lane == 0) {
    a.ncount[g] = n_acc;
    st4(mdisp, g, R4<R>{R(0), R(0), R(0), R(0)});
  }
}

// One warp per bead, the warps striding over the beads.
template <typename R>
__global__ void __launch_bounds__(PMD_NT)
    k_pmd_nlist(PmdArgs a, const RepInfo* reps, const R* pos, R* mdisp, int adv_k,
                double adv_scale) {
  pmd_wait_previous();
  const int s = adv_k & 1;
  const RepInfo& ri = reps[a.rep];
  if (a.flag[s] == 0) return;
  __shared__ int s_buf[PMD_NT / 32][PMD_NL_CAP];
  const int warp = static_cast<int>(threadIdx.x) >> 5, lane = static_cast<int>(threadIdx.x) & 31;
  const PmdBox<R> b = pmd_box<R>(ri, a.dl_slot[s]);
  const R rv2 = static_cast<R>(ri.r_verlet) * static_cast<R>(ri.r_verlet);
  for (int i = static_cast<int>(blockIdx.x) * (PMD_NT / 32) + warp; i < a.n;
       i += static_cast<int>(gridDim.x) * (PMD_NT / 32)) {
    pmd_list_bead(a, s, b, rv2, pos, mdisp, i, lane, s_buf[warp]);
    __syncwarp();  // the buffer is refilled by the warp's next bead
  }
}

// Substep k: forces at positions pin, second half kick; with drift_next,
// substep k+1's kick, drift, wrap and binning into pout.
template <typename R, int LANES>
__global__ void __launch_bounds__(PMD_NT)
    k_pmd_forces(PmdArgs a, const RepInfo* reps, RepDyn* dyn, const R* pin, R* pout, R* mvel,
                 R* mfrc, R* mdisp, int adv_k, double adv_scale, int kick, int drift_next,
                 int calc_epot) {
  static_assert(32 % LANES == 0 && LANES <= PMD_MAX_LANES, "lanes of a bead within one warp");
  pmd_wait_previous();
  const RepInfo& ri = reps[a.rep];
  const int s = adv_k & 1;
  const PmdBox<R> b = pmd_box<R>(ri, a.dl_slot[s]);
  const int t = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
  const int i = t / LANES, sub = t % LANES;
  double ep = 0.0;
  R F0 = R(0), F1 = R(0), F2 = R(0);
  size_t g = 0;
  R4<R> x{}, v{};
  if (i < a.n) {
    const R lambda = static_cast<R>(ri.lambda);
    const int pot = ri.potential;
    g = static_cast<size_t>(a.base) + i;
    x = ld4_rw(pin, g);
    const bool ai = a.amphi[g] != 0;
    const int cnt = a.ncount[g];
    const int* nl = a.nlist + static_cast<size_t>(i) * a.max_nb;
    // (Box.cpp:243-286) pairs in index order (every LANES-th to each lane),
    // four independent neighbour loads at a time; then the bead's bonds
    constexpr int PF = 4;
    for (int q0 = sub; q0 < cnt; q0 += PF * LANES) {
      int js[PF];
#pragma unroll
      for (int u = 0; u < PF; ++u) {
        const int q = q0 + u * LANES;
        js[u] = q < cnt ? nl[q] : -1;
      }
#pragma unroll
      for (int u = 0; u < PF; ++u) {
        const int j = js[u];
        if (j < 0) continue;
        const R4<R> y = ld4_rw(pin, static_cast<size_t>(j));
        R d0 = y.x - x.x, d1 = y.y - x.y, d2 = y.z - x.z;
        pmd_min_image(d0, d1, d2, b);
        const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
        const bool bb = ai && a.amphi[j] != 0;
        const R fa = pair_force<R>(pot, bb, r2, lambda);
        F0 -= d0 * fa;
        F1 -= d1 * fa;
        F2 -= d2 * fa;
        if (calc_epot) ep += 0.5 * static_cast<double>(pair_pot<R>(pot, bb, r2, lambda));
      }
    }
    for (int e = a.bond_start[g] + sub; e < a.bond_start[g + 1]; e += LANES) {
      const int2 bd = a.bonds[e];
      const R4<R> y = ld4_rw(pin, static_cast<size_t>(bd.x));
      R d0 = y.x - x.x, d1 = y.y - x.y, d2 = y.z - x.z;
      pmd_min_image(d0, d1, d2, b);
      const bool anch = bd.y != 0;
      R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
      if (pot == POT_REF4824) {
        // reference FENE: beyond R0 the force changes sign (Potentials.h:24-55)
        if (r2 >= (anch ? R(20.25) : R(2.25)))
          raise_error(a.err, ERR_FENE, static_cast<uint32_t>(g), static_cast<uint32_t>(bd.x));
      } else {
        const R cap = (anch ? R(20.25) : R(2.25)) * R(0.98);
        if (r2 > cap) r2 = cap;
      }
      const R fa = fene_force<R>(anch, r2);
      F0 -= d0 * fa;
      F1 -= d1 * fa;
      F2 -= d2 * fa;
      if (calc_epot) ep += 0.5 * static_cast<double>(fene_pot<R>(anch, r2));
    }
  }
  // the lanes of a bead are adjacent within one warp (LANES divides 32)
  for (int o = 1; o < LANES; o <<= 1) {
    F0 += __shfl_xor_sync(0xFFFFFFFFu, F0, o);
    F1 += __shfl_xor_sync(0xFFFFFFFFu, F1, o);
    F2 += __shfl_xor_sync(0xFFFFFFFFu, F2, o);
  }
  if (i < a.n && sub == 0) {
    st4(mfrc, g, R4<R>{F0, F1, F2, R(0)});
    // this substep's grid is empty again: its beads' cells back to zero
    a.cnt[s][pmd_cell(a, b, x)] = 0u;
    v = ld4_rw(mvel, g);
    if (kick) {  // second half kick (Thermostat_None.cpp:33-37)
      const R dth = static_cast<R>(ri.md_dt) * R(0.50);
      v.x += pmd_kick(F0, x.w, dth, a.andersen);
      v.y += pmd_kick(F1, x.w, dth, a.andersen);
      v.z += pmd_kick(F2, x.w, dth, a.andersen);
      if (a.andersen) {
        R w[3] = {v.x, v.y, v.z};
        andersen_draw<R>(ri.seed, i, dyn[a.rep].md_step, static_cast<R>(a.andersen_nu * ri.md_dt),
                         r_sqrt(static_cast<R>(ri.kT)), x.w, w);
        v.x = w[0];
        v.y = w[1];
        v.z = w[2];
      }
    }
    if (drift_next) {
      const PmdBox<R> b1 = pmd_box<R>(ri, a.dl_slot[s ^ 1]);
      R4<R> u = ld4_rw(mdisp, g);
      pmd_drift_bead(ri, b1, x, v, u, F0, F1, F2, a.andersen);
      pmd_wrap(ri, b1, x, v);
      st4(pout, g, x);
      st4(mdisp, g, u);
      pmd_bin(a, s ^ 1, b1, x, i);
      const R thr = static_cast<R>(a.dl_slot[2 + (s ^ 1)]);
      if (thr <= R(0) || (u.x * u.x + u.y * u.y) + u.z * u.z > thr * thr) a.flag[s ^ 1] = 1;
    }
    if (kick || drift_next) st4(mvel, g, v);
  }
  if (calc_epot) {
    __shared__ double s_red[PMD_NT / 32];
    const double tot = block_sum<PMD_NT>(ep, s_red);
    if (threadIdx.x == 0) a.epot_part[blockIdx.x] = tot;
  }
  // the last block to get here closes the substep (no block waits for another)
  if (!pmd_last_block(a)) return;
  RepDyn& dn = dyn[a.rep];
  if (kick) dn.md_step += 1;  // the thermostat's draws of this substep are done
  if (a.flag[s] != 0) {
    *a.delrx_build = a.dl_slot[s];
    a.flag[3] = 0;
    dn.verlet_rebuilds += 1;
  } else {
    a.flag[3] += 1;
  }
  a.flag[s] = 0;
  if (calc_epot) {
    double tot = 0.0;
    for (int k = 0; k < static_cast<int>(gridDim.x); ++k) tot += a.epot_part[k];
    dn.epot = tot;
  }
  // the next substep's request is final too: the constants of the one after
  pmd_next_constants<R>(a, ri, s ^ 1, adv_scale);
}

template <typename R>
__global__ void __launch_bounds__(PMD_NT) k_pmd_copy(PmdArgs a, const R* src, R* dst) {
  pmd_wait_previous();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const size_t g = static_cast<size_t>(a.base) + i;
  st4(dst, g, ld4_rw(src, g));
}

}  // namespace smpc
