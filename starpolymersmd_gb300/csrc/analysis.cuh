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
//                    sum_i v_i(oldest) . v_i(oldest + j) over the window.
// Positions and velocities are the stored ones (primary box after a
// collision), as the functors read Particle::Position / Velocity.
#pragma once
#include <stdint.h>

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
