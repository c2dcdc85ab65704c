// Solvent analyses of the reference's Analysis functors, with the sums over
// particles on the device (FP64 accumulation, per-block partials summed in
// block order, so results do not depend on scheduling):
//   k_fourier_modes  Fourier_Autocorr::operator() (Fourier_Autocorr.h): for
//                    k = (2 pi / L) e_j, j = x, y, z, the mode
//                    sum_i v_i exp(i k . r_i); the host divides by N and
//                    removes the component along k;
//   k_vacf_sample    Vel_Autocorr_Fluid::operator() (Vel_Autocorr_Fluid.h):
//                    the velocities of solvent particles 0..N_p-1 into slot
//                    s of a ring of `entries` samples;
//   k_vacf_lags      Vel_Autocorr_Fluid::calculate(): for every lag j,
//                    sum_i v_i(oldest) . v_i(oldest + j) over the window;
//   k_kinetic_tensor, k_mono_stress  the pressure tensor (no reference
//                    counterpart; below).
// Positions and velocities are the stored ones (primary box after a
// collision), as the functors read Particle::Position / Velocity.
#pragma once
#include <stdint.h>

#include "md_kernels.cuh"
#include "mpc_kernels.cuh"
#include "observables.cuh"

namespace smpc {

constexpr int ANA_NT = 256;

// One block per tile of solvent slots; part[18 * block]: the three modes
// (x, y, z components of k_x, then k_y, k_z), (re, im) interleaved.
template <typename R>
__global__ void __launch_bounds__(ANA_NT)
    k_fourier_modes(const RepInfo* reps, int rep, const R* rec, double kwave, double* part) {
  __shared__ double s_red[ANA_NT / 32];
  const RepInfo& ri = reps[rep];
  double acc[18];
#pragma unroll
  for (int q = 0; q < 18; ++q) acc[q] = 0.0;
  for (int i = blockIdx.x * ANA_NT + threadIdx.x; i < ri.slot_cap; i += gridDim.x * ANA_NT) {
    const size_t s = static_cast<size_t>(ri.slot_base) + i;
    const R* p = rec + 8 * s;
    if (slot_id(p[3]) == SLOT_EMPTY) continue;
    const double v[3] = {static_cast<double>(p[4]), static_cast<double>(p[5]),
                         static_cast<double>(p[6])};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double sn, cs;
      sincos(kwave * static_cast<double>(p[j]), &sn, &cs);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        acc[6 * j + 2 * d] += v[d] * cs;
        acc[6 * j + 2 * d + 1] += v[d] * sn;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 18; ++q) {
    const double t = block_sum<ANA_NT>(acc[q], s_red);
    if (threadIdx.x == 0) part[18 * static_cast<size_t>(blockIdx.x) + q] = t;
  }
}

// ring[(slot * n_p + id) * 3 + d] <- v_d of solvent particle id < n_p
template <typename R>
__global__ void __launch_bounds__(ANA_NT)
    k_vacf_sample(const RepInfo* reps, int rep, const R* rec, int n_p, int slot, double* ring) {
  const RepInfo& ri = reps[rep];
  for (int i = blockIdx.x * ANA_NT + threadIdx.x; i < ri.slot_cap; i += gridDim.x * ANA_NT) {
    const R* p = rec + 8 * (static_cast<size_t>(ri.slot_base) + i);
    const uint32_t id = slot_id(p[3]);
    if (id == SLOT_EMPTY || id >= static_cast<uint32_t>(n_p)) continue;
    double* r = ring + (static_cast<size_t>(slot) * n_p + id) * 3;
    r[0] = static_cast<double>(p[4]);
    r[1] = static_cast<double>(p[5]);
    r[2] = static_cast<double>(p[6]);
  }
}

// blockIdx.y = lag j; blocks along x stride over the particles.
// part[j * gridDim.x + blockIdx.x] = sum over its particles of
// v(oldest) . v(oldest + j); slot of window position q = (first + q) % entries.
template <typename R>  // R: the instantiating unit's precision (one copy per unit)
__global__ void __launch_bounds__(ANA_NT)
    k_vacf_lags(const double* ring, int n_p, int entries, int first, double* part) {
  __shared__ double s_red[ANA_NT / 32];
  const int j = blockIdx.y;
  const size_t s0 = static_cast<size_t>(first % entries) * n_p;
  const size_t sj = static_cast<size_t>((first + j) % entries) * n_p;
  double acc = 0.0;
  for (int i = blockIdx.x * ANA_NT + threadIdx.x; i < n_p; i += gridDim.x * ANA_NT) {
    const double* a = ring + (s0 + i) * 3;
    const double* b = ring + (sj + i) * 3;
    acc += (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
  }
  const double t = block_sum<ANA_NT>(acc, s_red);
  if (threadIdx.x == 0) part[static_cast<size_t>(j) * gridDim.x + blockIdx.x] = t;
}

}  // namespace smpc

namespace smpc {

// ------------------------------------------------------------ pressure tensor
// P = (1/V) [sum_i m u_i u_i^T + sum over pairs r_ij F_ij^T]: the kinetic part
// with the peculiar velocity u = v - shear y e_x (the Lees-Edwards flow removed,
// y in the box frame) and the monomers' pair and FENE virial (each pair and
// bond once: half of the per-bead sums over both ends). No reference
// computes it; the MPC collision's momentum transfer is not included.
// Components xx yy zz xy xz yz.

__device__ __forceinline__ void stress_add(double* t, double a0, double a1, double a2, double b0,
                                           double b1, double b2, double w) {
  t[0] += w * a0 * b0;
  t[1] += w * a1 * b1;
  t[2] += w * a2 * b2;
  t[3] += w * a0 * b1;
  t[4] += w * a0 * b2;
  t[5] += w * a1 * b2;
}

// solvent: one block per tile of slots, part[6 * tile]
template <typename R>
__global__ void __launch_bounds__(ANA_NT)
    k_kinetic_tensor(const Tile* tiles, const RepInfo* reps, const R* rec, double* part) {
  __shared__ double s_red[ANA_NT / 32];
  const Tile t = tiles[blockIdx.x];
  const RepInfo& ri = reps[t.rep];
  const double m = ri.solvent_mass;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int i = t.begin + threadIdx.x; i < t.end; i += ANA_NT) {
    const R* p = rec + 8 * static_cast<size_t>(i);
    if (slot_id(p[3]) == SLOT_EMPTY) continue;
    const double u0 = static_cast<double>(p[4]) - ri.shear * static_cast<double>(p[1]);
    const double u1 = static_cast<double>(p[5]), u2 = static_cast<double>(p[6]);
    stress_add(acc, u0, u1, u2, u0, u1, u2, m);
  }
  for (int k = 0; k < 6; ++k) {
    const double s = block_sum<ANA_NT>(acc[k], s_red);
    if (threadIdx.x == 0) part[6 * static_cast<size_t>(blockIdx.x) + k] = s;
  }
}

// Monomers of one replica per block: kinetic part (6) and virial (6) into
// out[12 * r]. Periodic boxes: their row lists and the minimum image at the
// current delrx; other boxes: the transposed lists, plain differences.
template <typename R>
__global__ void __launch_bounds__(ANA_NT)
    k_mono_stress(const RepInfo* reps, const RepDyn* dyn, const R* mpos, const R* mvel,
                  const int* nlist_t, const int* ncount, int n_mono_total, int* const* rows,
                  int max_nb, const int* bond_start, const int2* bonds, double* out) {
  __shared__ double s_red[ANA_NT / 32];
  const int r = blockIdx.x;
  const RepInfo& ri = reps[r];
  const int* row = rows[r];
  const bool periodic = (ri.flags & REP_PERIODIC_MD) != 0;
  const double L[3] = {static_cast<double>(ri.L[0]), static_cast<double>(ri.L[1]),
                       static_cast<double>(ri.L[2])};
  const double delrx = dyn[r].delrx;
  const R lambda = static_cast<R>(ri.lambda);
  const int pot = ri.potential;
  double kin[6] = {0, 0, 0, 0, 0, 0}, vir[6] = {0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < ri.n_mono; i += ANA_NT) {
    const size_t g = static_cast<size_t>(ri.mono_base) + i;
    const R4<R> x = ld4_rw(mpos, g), v = ld4_rw(mvel, g);
    const double u0 = static_cast<double>(v.x) - ri.shear * static_cast<double>(x.y);
    stress_add(kin, u0, v.y, v.z, u0, v.y, v.z, static_cast<double>(x.w));
    const bool ai = (static_cast<int>(v.w) & 1) != 0;
    auto pair_vec = [&](size_t j, double* d) {
      const R4<R> y = ld4_rw(mpos, j);
      d[0] = static_cast<double>(y.x) - static_cast<double>(x.x);
      d[1] = static_cast<double>(y.y) - static_cast<double>(x.y);
      d[2] = static_cast<double>(y.z) - static_cast<double>(x.z);
      if (periodic) {
        const double cy = round(d[1] / L[1]);
        d[0] -= L[0] * round(d[0] / L[0]);
        d[0] -= cy * delrx;
        d[0] -= L[0] * round(d[0] / L[0]);
        d[1] -= L[1] * cy;
        d[2] -= L[2] * round(d[2] / L[2]);
      }
    };
    const int cnt = ncount[g];
    for (int q = 0; q < cnt; ++q) {
      const int j = row ? row[static_cast<size_t>(i) * max_nb + q]
                        : nlist_t[static_cast<size_t>(q) * n_mono_total + g];
      double d[3];
      pair_vec(static_cast<size_t>(j), d);
      const double r2 = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
      const bool bb = ai && (static_cast<int>(mvel[4 * static_cast<size_t>(j) + 3]) & 1) != 0;
      const double fa = static_cast<double>(pair_force<R>(pot, bb, static_cast<R>(r2), lambda));
      stress_add(vir, d[0], d[1], d[2], d[0], d[1], d[2], 0.5 * fa);
    }
    for (int e = bond_start[g]; e < bond_start[g + 1]; ++e) {
      const int2 bd = bonds[e];
      double d[3];
      pair_vec(static_cast<size_t>(bd.x), d);
      R r2 = static_cast<R>((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
      const bool anch = bd.y != 0;
      if (pot != POT_REF4824) {
        const R cap = (anch ? R(20.25) : R(2.25)) * R(0.98);
        if (r2 > cap) r2 = cap;
      }
      const double fa = static_cast<double>(fene_force<R>(anch, r2));
      stress_add(vir, d[0], d[1], d[2], d[0], d[1], d[2], 0.5 * fa);
    }
  }
  for (int k = 0; k < 6; ++k) {
    const double a = block_sum<ANA_NT>(kin[k], s_red);
    const double b = block_sum<ANA_NT>(vir[k], s_red);
    if (threadIdx.x == 0) {
      out[12 * static_cast<size_t>(r) + k] = a;
      out[12 * static_cast<size_t>(r) + 6 + k] = b;
    }
  }
}

}  // namespace smpc
