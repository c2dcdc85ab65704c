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
// One substep of one periodic box is five launches over its beads:
//   k_pmd_drift   half kick and drift, Lees-Edwards wrap, displacement since
//                 the last list build, rebuild request
//   k_pmd_bin     (rebuild only) beads into fixed-capacity grid cells
//   k_pmd_nlist   (rebuild only) Verlet lists from the 27 neighbour cells;
//                 across a y face the neighbour rows are looked up at x -/+
//                 delrx. Each list is kept in bead-index order, so the force
//                 sums do not depend on the order the atomics binned in.
//   k_pmd_forces  forces and the second half kick; empties the grid after a
//                 rebuild
//   k_pmd_finish  records the new lists' delrx, clears the request, sums the
//                 potential energy of the blocks in a fixed order
// A rebuild is requested when a bead has moved more than half of what is left
// of the skin after the change of delrx since the last build: pairs across the
// y faces see that change as a relative displacement. For periodic boxes the
// Verlet-reference array holds that displacement (summed v dt), which wrapping
// does not disturb.
#pragma once
#include <stdint.h>

#include "md_kernels.cuh"
#include "observables.cuh"

namespace smpc {

constexpr int PMD_CELL_CAP = 128;  // beads per grid cell
constexpr int PMD_NT = 256;        // threads per block of every periodic-MD kernel

struct PmdArgs {
  int rep;
  int base;            // first global monomer of the box
  int n;               // beads
  int nc[3];           // grid cells per axis (>= 3, side >= r_verlet)
  int ncell;
  int n_blocks;        // blocks of the per-bead launches
  uint32_t* cnt;       // beads per grid cell; zero between rebuilds
  int* items;          // ncell x PMD_CELL_CAP bead indices (box-local)
  int* flag;           // rebuild requested
  double* delrx_build; // delrx of the current lists
  double* epot_part;   // per block of k_pmd_forces
  int* nlist;          // [max_nb][n_mono_total] global indices, as md_kernels.cuh
  int* ncount;
  int n_mono_total;
  int max_nb;
  const int* bond_start;
  const int2* bonds;
  ErrorState* err;
};

// delrx after k more MD steps: k_cycle_begin's operations (MPC.cpp:117-118)
__device__ __forceinline__ double pmd_delrx(const RepInfo& ri, double d, int k,
                                            double adv_scale) {
  const double Lx = static_cast<double>(ri.L[0]);
  const double adv_dt = __dmul_rn(ri.h, adv_scale);
  for (int s = 0; s < k; ++s) {
    d = __dadd_rn(d, __dmul_rn(__dmul_rn(ri.shear, static_cast<double>(ri.L[1])), adv_dt));
    d = __dsub_rn(d, __dmul_rn(Lx, round(__ddiv_rn(d, Lx))));
  }
  return d;
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

// Lees-Edwards minimum image of d = x_j - x_i (MPC::relative_position)
template <typename R>
__device__ __forceinline__ void pmd_min_image(R& dx, R& dy, R& dz, const PmdBox<R>& b) {
  const R cy = r_round(pmd_ratio(dy, b.L[1], b.inv[1]));
  dx -= b.L[0] * r_round(pmd_ratio(dx, b.L[0], b.inv[0]));
  dx -= cy * b.delrx;
  dx -= b.L[0] * r_round(pmd_ratio(dx, b.L[0], b.inv[0]));
  dy -= b.L[1] * cy;
  dz -= b.L[2] * r_round(pmd_ratio(dz, b.L[2], b.inv[2]));
}

template <typename R>
__device__ __forceinline__ int pmd_cell_axis(R x, R L, int nc) {
  const int c = static_cast<int>(r_floor((x + R(0.5) * L) * (static_cast<R>(nc) / L)));
  return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

// delrx of this launch's substep, computed once per block
__device__ __forceinline__ double pmd_block_delrx(const RepInfo& ri, const RepDyn* dyn, int rep,
                                                  int adv_k, double adv_scale) {
  __shared__ double s_dl;
  if (threadIdx.x == 0) s_dl = pmd_delrx(ri, dyn[rep].delrx, adv_k, adv_scale);
  __syncthreads();
  return s_dl;
}

template <typename R>
__global__ void __launch_bounds__(PMD_NT)
    k_pmd_drift(PmdArgs a, const RepInfo* reps, const RepDyn* dyn, R* mpos, R* mvel,
                const R* mfrc, R* mdisp, int adv_k, double adv_scale, int drift) {
  const RepInfo& ri = reps[a.rep];
  const double dl = pmd_block_delrx(ri, dyn, a.rep, adv_k, adv_scale);
  __shared__ R s_thr;
  if (threadIdx.x == 0) {
    const double Lx = static_cast<double>(ri.L[0]);
    double ddl = dl - *a.delrx_build;
    ddl -= Lx * round(ddl / Lx);
    s_thr = static_cast<R>(0.5 * ((ri.r_verlet - ri.r_cut) - fabs(ddl)));
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const PmdBox<R> b = pmd_box<R>(ri, dl);
  const size_t g = static_cast<size_t>(a.base) + i;
  R4<R> x = ld4_rw(mpos, g), v = ld4_rw(mvel, g), u = ld4_rw(mdisp, g);
  if (drift) {
    const R4<R> f = ld4_rw(mfrc, g);
    const R dt = static_cast<R>(ri.md_dt), dth = dt * R(0.50);
    // kick + drift (Thermostat_None.cpp:22-27)
    v.x += (f.x / x.w) * dth;
    x.x += v.x * dt;
    u.x += v.x * dt;
    v.y += (f.y / x.w) * dth;
    x.y += v.y * dt;
    u.y += v.y * dt;
    v.z += (f.z / x.w) * dth;
    x.z += v.z * dt;
    u.z += v.z * dt;
  }
  // back into the primary box (MPC::LEBC); the set-up call (drift = 0) only
  // wraps what the caller placed outside
  const R cy = r_round(pmd_ratio(x.y, b.L[1], b.inv[1]));
  x.x -= b.L[0] * r_round(pmd_ratio(x.x, b.L[0], b.inv[0]));
  x.x -= cy * b.delrx;
  x.x -= b.L[0] * r_round(pmd_ratio(x.x, b.L[0], b.inv[0]));
  x.y -= b.L[1] * cy;
  x.z -= b.L[2] * r_round(pmd_ratio(x.z, b.L[2], b.inv[2]));
  v.x -= cy * static_cast<R>(ri.shear) * b.L[1];
  st4(mpos, g, x);
  st4(mvel, g, v);
  if (!drift) {  // set-up: lists and forces from the current positions
    if (i == 0) *a.flag = 1;
    return;
  }
  st4(mdisp, g, u);
  const R thr = s_thr;
  if (thr <= R(0) || (u.x * u.x + u.y * u.y) + u.z * u.z > thr * thr) *a.flag = 1;
}

template <typename R>
__global__ void __launch_bounds__(PMD_NT) k_pmd_bin(PmdArgs a, const RepInfo* reps, const R* mpos) {
  if (*a.flag == 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const RepInfo& ri = reps[a.rep];
  const R4<R> x = ld4_rw(mpos, static_cast<size_t>(a.base) + i);
  const int cx = pmd_cell_axis(x.x, static_cast<R>(ri.L[0]), a.nc[0]);
  const int cy = pmd_cell_axis(x.y, static_cast<R>(ri.L[1]), a.nc[1]);
  const int cz = pmd_cell_axis(x.z, static_cast<R>(ri.L[2]), a.nc[2]);
  const int c = cx + a.nc[0] * (cy + a.nc[1] * cz);
  const uint32_t k = atomicAdd(a.cnt + c, 1u);
  if (k < static_cast<uint32_t>(PMD_CELL_CAP))
    a.items[static_cast<size_t>(c) * PMD_CELL_CAP + k] = i;
  else
    raise_error(a.err, ERR_NEIGHBOR_OVF, static_cast<uint32_t>(a.base + i), k);
}

template <typename R>
__global__ void __launch_bounds__(PMD_NT)
    k_pmd_nlist(PmdArgs a, const RepInfo* reps, const RepDyn* dyn, const R* mpos, R* mdisp,
                int adv_k, double adv_scale) {
  if (*a.flag == 0) return;
  const RepInfo& ri = reps[a.rep];
  const PmdBox<R> b = pmd_box<R>(ri, pmd_block_delrx(ri, dyn, a.rep, adv_k, adv_scale));
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const R rv2 = static_cast<R>(ri.r_verlet) * static_cast<R>(ri.r_verlet);
  const size_t g = static_cast<size_t>(a.base) + i;
  const R4<R> x = ld4_rw(mpos, g);
  const int nx = a.nc[0], ny = a.nc[1], nz = a.nc[2];
  const int cy = pmd_cell_axis(x.y, b.L[1], ny);
  const int cz = pmd_cell_axis(x.z, b.L[2], nz);
  const size_t stride = static_cast<size_t>(a.n_mono_total);
  int* nl = a.nlist + g;
  int cnt = 0;
  for (int oz = -1; oz <= 1; ++oz) {
    const int zz = (cz + oz + nz) % nz;
    for (int oy = -1; oy <= 1; ++oy) {
      const int yr = cy + oy;
      const int yy = (yr + ny) % ny;
      // the row beyond a y face is the image shifted by delrx along x
      R xc = x.x;
      if (yr >= ny) xc -= b.delrx;
      if (yr < 0) xc += b.delrx;
      xc -= b.L[0] * r_round(pmd_ratio(xc, b.L[0], b.inv[0]));
      const int cx = pmd_cell_axis(xc, b.L[0], nx);
      for (int ox = -1; ox <= 1; ++ox) {
        const int c = (cx + ox + nx) % nx + nx * (yy + ny * zz);
        const int m = min(static_cast<int>(a.cnt[c]), PMD_CELL_CAP);
        for (int q = 0; q < m; ++q) {
          const int j = a.items[static_cast<size_t>(c) * PMD_CELL_CAP + q];
          if (j == i) continue;
          const R4<R> y = ld4_rw(mpos, static_cast<size_t>(a.base) + j);
          R d0 = y.x - x.x, d1 = y.y - x.y, d2 = y.z - x.z;
          pmd_min_image(d0, d1, d2, b);
          if ((d0 * d0 + d1 * d1) + d2 * d2 <= rv2) {
            if (cnt < a.max_nb) {  // insertion in index order
              int p = cnt;
              while (p > 0 && nl[static_cast<size_t>(p - 1) * stride] > a.base + j) {
                nl[static_cast<size_t>(p) * stride] = nl[static_cast<size_t>(p - 1) * stride];
                --p;
              }
              nl[static_cast<size_t>(p) * stride] = a.base + j;
            }
            ++cnt;
          }
        }
      }
    }
  }
  if (cnt > a.max_nb) {
    raise_error(a.err, ERR_NEIGHBOR_OVF, static_cast<uint32_t>(g), static_cast<uint32_t>(cnt));
    cnt = a.max_nb;
  }
  a.ncount[g] = cnt;
  st4(mdisp, g, R4<R>{R(0), R(0), R(0), R(0)});
}

template <typename R>
__global__ void __launch_bounds__(PMD_NT)
    k_pmd_forces(PmdArgs a, const RepInfo* reps, const RepDyn* dyn, const R* mpos, R* mvel,
                 R* mfrc, int adv_k, double adv_scale, int kick, int calc_epot) {
  const RepInfo& ri = reps[a.rep];
  const PmdBox<R> b = pmd_box<R>(ri, pmd_block_delrx(ri, dyn, a.rep, adv_k, adv_scale));
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ep = 0.0;
  if (i < a.n) {
    const R lambda = static_cast<R>(ri.lambda);
    const int pot = ri.potential;
    const size_t g = static_cast<size_t>(a.base) + i;
    const R4<R> x = ld4_rw(mpos, g);
    R4<R> v = ld4_rw(mvel, g);
    const bool ai = (static_cast<int>(v.w) & 1) != 0;
    const size_t stride = static_cast<size_t>(a.n_mono_total);
    R F0 = R(0), F1 = R(0), F2 = R(0);
    const int cnt = a.ncount[g];
    const int* nl = a.nlist + g;
    // (Box.cpp:243-286) pairs in index order, then the bead's bonds; the
    // neighbour indices come four at a time, as independent loads
    constexpr int PF = 4;
    for (int q0 = 0; q0 < cnt; q0 += PF) {
      int js[PF];
#pragma unroll
      for (int u = 0; u < PF; ++u)
        js[u] = q0 + u < cnt ? nl[static_cast<size_t>(q0 + u) * stride] : -1;
#pragma unroll
      for (int u = 0; u < PF; ++u) {
        const int j = js[u];
        if (j < 0) continue;
        const R4<R> y = ld4_rw(mpos, static_cast<size_t>(j));
        const R wy = mvel[4 * static_cast<size_t>(j) + 3];
        R d0 = y.x - x.x, d1 = y.y - x.y, d2 = y.z - x.z;
        pmd_min_image(d0, d1, d2, b);
        const R r2 = (d0 * d0 + d1 * d1) + d2 * d2;
        const bool bb = ai && (static_cast<int>(wy) & 1) != 0;
        const R fa = pair_force<R>(pot, bb, r2, lambda);
        F0 -= d0 * fa;
        F1 -= d1 * fa;
        F2 -= d2 * fa;
        if (calc_epot) ep += 0.5 * static_cast<double>(pair_pot<R>(pot, bb, r2, lambda));
      }
    }
    for (int e = a.bond_start[g]; e < a.bond_start[g + 1]; ++e) {
      const int2 bd = a.bonds[e];
      const R4<R> y = ld4_rw(mpos, static_cast<size_t>(bd.x));
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
    st4(mfrc, g, R4<R>{F0, F1, F2, R(0)});
    if (kick) {  // second half kick (Thermostat_None.cpp:33-37)
      const R dth = static_cast<R>(ri.md_dt) * R(0.50);
      v.x += (F0 / x.w) * dth;
      v.y += (F1 / x.w) * dth;
      v.z += (F2 / x.w) * dth;
      st4(mvel, g, v);
    }
  }
  if (calc_epot) {
    __shared__ double s_red[PMD_NT / 32];
    const double t = block_sum<PMD_NT>(ep, s_red);
    if (threadIdx.x == 0) a.epot_part[blockIdx.x] = t;
  }
  if (*a.flag != 0) {  // the grid is empty again for the next rebuild
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.ncell; c += gridDim.x * blockDim.x)
      a.cnt[c] = 0u;
  }
}

template <typename R>
__global__ void k_pmd_finish(PmdArgs a, const RepInfo* reps, RepDyn* dyn, int adv_k,
                             double adv_scale, int calc_epot) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  RepDyn& dn = dyn[a.rep];
  if (*a.flag != 0) {
    *a.delrx_build = pmd_delrx(reps[a.rep], dn.delrx, adv_k, adv_scale);
    *a.flag = 0;
    dn.verlet_rebuilds += 1;
  }
  if (calc_epot) {
    double s = 0.0;
    for (int k = 0; k < a.n_blocks; ++k) s += a.epot_part[k];
    dn.epot = s;
  }
}

}  // namespace smpc
