// Output-step observables on the device, FP64 (star-polymers.cpp:466-483):
//   k_mol_observables  per replica: radius of gyration and gyration tensor
//                      (Box::calculate_gyration_tensor, Box.cpp:330-353),
//                      rotation frequency (Box::calculate_rotation_frequency,
//                      Box.cpp:355-379), kinetic energy and temperature
//                      (Box::calculate_ekin / print_Ekin_and_Temperature,
//                      Box.cpp:288-294, 635-646), all in each molecule's
//                      centre-of-mass frame (Box::center_of_mass_reference_frame,
//                      Box.cpp:81-102);
//   k_velocity_profile VelocityX (Velocity_x.h:76-100): solvent velocity
//                      relative to molecule 0's centre-of-mass velocity, binned
//                      by the Lees-Edwards-wrapped position relative to its
//                      centre of mass, along x and along y.
// Centres of mass are summed by one thread in monomer order, like the
// reference, so every position relative to them is the reference's to the
// last bit; the tensor, momentum and energy sums are block reductions.
#pragma once
#include <stdint.h>

#include <type_traits>

#include "mpc_kernels.cuh"
#include "smpc_device.cuh"

namespace smpc {

constexpr int OBS_PER_REP = 16;
constexpr int UNWRAP_NT = 256;  // threads (and beads per chunk) of k_unwrap_molecules

// centre of molecule [b, e): unweighted mean position and velocity
template <typename R>
__device__ __forceinline__ void molecule_centre(const R* mpos, const R* mvel, int b, int e,
                                                double* c) {
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int i = b; i < e; ++i) {
    const R4<R> p = ld4_rw(mpos, i), v = ld4_rw(mvel, i);
    s[0] += static_cast<double>(p.x);
    s[1] += static_cast<double>(p.y);
    s[2] += static_cast<double>(p.z);
    s[3] += static_cast<double>(v.x);
    s[4] += static_cast<double>(v.y);
    s[5] += static_cast<double>(v.z);
  }
  const double n = static_cast<double>(e - b);
  for (int k = 0; k < 6; ++k) c[k] = s[k] / n;
}

// x = A^-1 b for a symmetric positive-definite 3x3 A (LDL^T, no pivoting)
__device__ __forceinline__ void solve_sym3(const double A[3][3], const double b[3], double x[3]) {
  double L10 = 0, L20 = 0, L21 = 0, D0, D1, D2;
  D0 = A[0][0];
  L10 = A[1][0] / D0;
  L20 = A[2][0] / D0;
  D1 = A[1][1] - L10 * L10 * D0;
  L21 = (A[2][1] - L20 * L10 * D0) / D1;
  D2 = A[2][2] - L20 * L20 * D0 - L21 * L21 * D1;
  const double y0 = b[0];
  const double y1 = b[1] - L10 * y0;
  const double y2 = b[2] - L20 * y0 - L21 * y1;
  x[2] = y2 / D2;
  x[1] = y1 / D1 - L21 * x[2];
  x[0] = y0 / D0 - L10 * x[1] - L20 * x[2];
}

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* s_red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < NT / 32; ++w) t += s_red[w];
  return t;  // valid in thread 0
}

// K block sums at once, each with block_sum's order (so the same bits): one
// shuffle pass over all K values, one exchange, thread k < K adds the warps'
// partials of value k into out[k] (shared; valid in every thread on return).
// s_red holds K * NT / 32 doubles.
template <int NT, int K>
__device__ __forceinline__ void block_sum_n(double (&v)[K], double* s_red, double* out) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += __shfl_down_sync(0xFFFFFFFFu, v[k], o);
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) s_red[k * (NT / 32) + (threadIdx.x >> 5)] = v[k];
  __syncthreads();
  if (threadIdx.x < K) {
    double t = 0.0;
    for (int w = 0; w < NT / 32; ++w) t += s_red[threadIdx.x * (NT / 32) + w];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// One CTA per molecule; mols[m] = global monomer range [x, y). mol_out[16 m
// + ...]: R_g of the molecule, G (row-major, 9), rotation frequency (3),
// kinetic energy, monomers. FP64 sums the centre in monomer order (the
// reference's order, so the relative positions are the reference's to the
// last bit); FP32 sums it as a block reduction.
template <typename R, int NT>
__global__ void __launch_bounds__(NT) k_mol_observables(const int2* mols, const R* mpos,
                                                        const R* mvel, double* mol_out) {
  __shared__ double s_c[6];
  __shared__ double s_red[10 * (NT / 32)];
  __shared__ double s_tot[10];
  const int2 mb = mols[blockIdx.x];
  const int n = mb.y - mb.x;
  if (std::is_same<R, double>::value) {
    if (threadIdx.x == 0) molecule_centre<R>(mpos, mvel, mb.x, mb.y, s_c);
  } else {
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (int i = mb.x + threadIdx.x; i < mb.y; i += NT) {
      const R4<R> p = ld4_rw(mpos, i), v = ld4_rw(mvel, i);
      c[0] += static_cast<double>(p.x);
      c[1] += static_cast<double>(p.y);
      c[2] += static_cast<double>(p.z);
      c[3] += static_cast<double>(v.x);
      c[4] += static_cast<double>(v.y);
      c[5] += static_cast<double>(v.z);
    }
    block_sum_n<NT, 6>(c, s_red, s_tot);
    if (threadIdx.x < 6) s_c[threadIdx.x] = s_tot[threadIdx.x] / static_cast<double>(n);
  }
  __syncthreads();
  // S = sum r r^T (6), angular momentum (3), sum m |u|^2
  double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = mb.x + threadIdx.x; i < mb.y; i += NT) {
    const R4<R> p = ld4_rw(mpos, i), v = ld4_rw(mvel, i);
    const double x0 = static_cast<double>(p.x) - s_c[0], x1 = static_cast<double>(p.y) - s_c[1],
                 x2 = static_cast<double>(p.z) - s_c[2];
    const double u0 = static_cast<double>(v.x) - s_c[3], u1 = static_cast<double>(v.y) - s_c[4],
                 u2 = static_cast<double>(v.z) - s_c[5];
    acc[0] += x0 * x0;
    acc[1] += x0 * x1;
    acc[2] += x0 * x2;
    acc[3] += x1 * x1;
    acc[4] += x1 * x2;
    acc[5] += x2 * x2;
    acc[6] += x1 * u2 - x2 * u1;
    acc[7] += x2 * u0 - x0 * u2;
    acc[8] += x0 * u1 - x1 * u0;
    acc[9] += static_cast<double>(p.w) * ((u0 * u0 + u1 * u1) + u2 * u2);
  }
  block_sum_n<NT, 10>(acc, s_red, s_tot);
  if (threadIdx.x != 0) return;
  double tot[10];
  for (int k = 0; k < 10; ++k) tot[k] = s_tot[k];
  double* o = mol_out + static_cast<size_t>(OBS_PER_REP) * blockIdx.x;
  for (int k = 0; k < OBS_PER_REP; ++k) o[k] = 0.0;
  if (n <= 0) return;
  const double dn = static_cast<double>(n);
  double g[9];
  if (std::is_same<R, double>::value) {  // the reference's divisions (Box.cpp:330-379)
    const double gg[9] = {tot[0] / dn, tot[1] / dn, tot[2] / dn, tot[1] / dn, tot[3] / dn,
                          tot[4] / dn, tot[2] / dn, tot[4] / dn, tot[5] / dn};
    for (int k = 0; k < 9; ++k) g[k] = gg[k];
  } else {  // FP32 path: one division
    const double inv = 1.0 / dn;
    const double gg[9] = {tot[0] * inv, tot[1] * inv, tot[2] * inv, tot[1] * inv, tot[3] * inv,
                          tot[4] * inv, tot[2] * inv, tot[4] * inv, tot[5] * inv};
    for (int k = 0; k < 9; ++k) g[k] = gg[k];
  }
  for (int k = 0; k < 9; ++k) o[1 + k] = g[k];
  o[0] = sqrt(g[0] + g[4] + g[8]);
  const double tr = tot[0] + tot[3] + tot[5];
  const double I[3][3] = {{tr - tot[0], -tot[1], -tot[2]},
                          {-tot[1], tr - tot[3], -tot[4]},
                          {-tot[2], -tot[4], tr - tot[5]}};
  const double Lm[3] = {tot[6], tot[7], tot[8]};
  double om[3];
  solve_sym3(I, Lm, om);
  for (int k = 0; k < 3; ++k) o[10 + k] = om[k];
  o[13] = tot[9] * 0.5;
  o[14] = dn;
}

// One thread per replica: its molecules' values in molecule order. out[16 r
// + ...]: mean R_g, mean G (row-major, 9), mean rotation frequency (3),
// kinetic energy, temperature 2 E / (3 (N - 1)), molecules.
template <typename R>  // R: the precision of the instantiating unit (one copy per unit)
__global__ void k_obs_reduce(const int2* rep_mols, const double* mol_out, int n_rep, double* out) {
  // one warp per replica: lane l sums molecules l, l + 32, ... in order, then
  // a fixed xor butterfly joins the lanes (every lane ends with the same bits;
  // a replica of one molecule gets its values unchanged)
  constexpr unsigned FULL = 0xFFFFFFFFu;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n_rep) return;  // whole warps
  const int2 rm = rep_mols[r];
  double acc[14];  // R_g, G (9), rotation frequency (3), kinetic energy
#pragma unroll
  for (int k = 0; k < 14; ++k) acc[k] = 0.0;
  long long n_total = 0;
  for (int m = rm.x + lane; m < rm.x + rm.y; m += 32) {
    const double* o = mol_out + static_cast<size_t>(OBS_PER_REP) * m;
    double v[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) v[k] = o[k];
    if (v[14] <= 0.0) continue;
#pragma unroll
    for (int k = 0; k < 14; ++k) acc[k] += v[k];
    n_total += static_cast<long long>(v[14]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int k = 0; k < 14; ++k) acc[k] += __shfl_xor_sync(FULL, acc[k], off);
    n_total += __shfl_xor_sync(FULL, n_total, off);
  }
  if (lane != 0) return;
  const double nm = rm.y > 0 ? static_cast<double>(rm.y) : 1.0;
  double* o = out + static_cast<size_t>(OBS_PER_REP) * r;
  if (std::is_same<R, double>::value) {
    // the reference's divisions by Molecules.size() (Box.cpp:350-351, 378)
    o[0] = acc[0] / nm;
    for (int k = 0; k < 9; ++k) o[1 + k] = acc[1 + k] / nm;
    for (int k = 0; k < 3; ++k) o[10 + k] = acc[10 + k] / nm;
  } else {
    // FP32 path: one division (FP64 divisions are slow on this part); exact
    // for one molecule
    const double inv = 1.0 / nm;
    o[0] = acc[0] * inv;
    for (int k = 0; k < 9; ++k) o[1 + k] = acc[1 + k] * inv;
    for (int k = 0; k < 3; ++k) o[10 + k] = acc[10 + k] * inv;
  }
  o[13] = acc[13];
  o[14] = n_total > 1 ? acc[13] * 2. / (3. * static_cast<double>(n_total - 1)) : 0.0;
  o[15] = static_cast<double>(rm.y);
}

// Molecules of periodic boxes made whole for the observables: bead i is placed
// at the Lees-Edwards minimum image (MPC.cpp:456-465, current delrx) next to
// its lowest-indexed bonded partner in the molecule, which comes earlier and is
// already placed, or next to the molecule's first bead when it has none. Its
// v_x gets the shear velocity of the image it moved to (MPC.cpp:428).
// k_copy_monomers copies every monomer first; k_unwrap_molecules then runs one
// CTA per molecule of a periodic box over chunks of UNWRAP_NT beads: when
// every bead of a chunk has its partner either before the chunk (placed) or
// right before itself (stars and chains numbered outward from the core), the
// chunk is one segmented prefix sum of the bond vectors (warp scans joined in
// warp order); otherwise thread 0 walks it.
template <typename R>
__global__ void k_copy_monomers(int n, const R* mpos, const R* mvel, R* upos, R* uvel) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    st4(upos, i, ld4_rw(mpos, i));
    st4(uvel, i, ld4_rw(mvel, i));
  }
}

// Lees-Edwards minimum image of a bond vector. The image counts come from
// products with 1 / L: a bond is far shorter than half the box, so d / L is
// never near a half-integer and the count is the one the division gives.
__device__ __forceinline__ void unwrap_bond(const double L[3], const double invL[3], double delrx,
                                            double& d0, double& d1, double& d2) {
  const double cy = round(d1 * invL[1]);
  d0 -= L[0] * round(d0 * invL[0]);
  d0 -= cy * delrx;
  d0 -= L[0] * round(d0 * invL[0]);
  d1 -= L[1] * cy;
  d2 -= L[2] * round(d2 * invL[2]);
}

template <typename R>
__global__ void __launch_bounds__(UNWRAP_NT)
    k_unwrap_molecules(const RepInfo* reps, const RepDyn* dyn, const int2* mols,
                       const int* mol_rep, int n_mols, const int* bond_start, const int2* bonds,
                       const R* mpos, const R* mvel, R* upos, R* uvel) {
  constexpr unsigned FULL = 0xFFFFFFFFu;
  constexpr int NW = UNWRAP_NT / 32;
  __shared__ double s_wsum[3][NW];  // per warp: the scan value of its last lane
  __shared__ int s_whead[NW];       // per warp: it holds a segment head
  __shared__ double s_carry[3][NW];  // per warp: what its leading (headless) lanes add
  __shared__ int s_walk;            // the chunk needs the one-by-one walk
  __shared__ int s_p[UNWRAP_NT];
  __shared__ double s_d[3][UNWRAP_NT];
  const int m = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const RepInfo& ri = reps[mol_rep[m]];
  if (!(ri.flags & REP_PERIODIC_MD)) return;  // whole block
  const double L[3] = {static_cast<double>(ri.L[0]), static_cast<double>(ri.L[1]),
                       static_cast<double>(ri.L[2])};
  const double invL[3] = {1.0 / L[0], 1.0 / L[1], 1.0 / L[2]};
  const double delrx = dyn[mol_rep[m]].delrx;
  const double sLy = ri.shear * L[1];
  const int2 mb = mols[m];
  for (int c0 = mb.x + 1; c0 < mb.y; c0 += UNWRAP_NT) {
    const int i = c0 + tid;
    const bool active = i < mb.y;
    int p = -1;
    double d0 = 0, d1 = 0, d2 = 0, xy = 0, uy = 0;
    if (tid == 0) s_walk = 0;
    if (active) {
      for (int e = bond_start[i]; e < bond_start[i + 1]; ++e) {
        const int j = bonds[e].x;
        if (j >= mb.x && j < i && (p < 0 || j < p)) p = j;
      }
      if (p < 0) p = mb.x;
      const R4<R> x = ld4_rw(mpos, i), xp = ld4_rw(mpos, p);
      xy = static_cast<double>(x.y);
      d0 = static_cast<double>(x.x) - static_cast<double>(xp.x);
      d1 = xy - static_cast<double>(xp.y);
      d2 = static_cast<double>(x.z) - static_cast<double>(xp.z);
      unwrap_bond(L, invL, delrx, d0, d1, d2);
    }
    const bool chained = active && p == i - 1 && p >= c0;
    __syncthreads();
    if (active && p >= c0 && !chained) s_walk = 1;
    __syncthreads();
    if (s_walk) {
      // a partner inside the chunk that is not the previous bead: one by one
      s_p[tid] = p;
      s_d[0][tid] = d0;
      s_d[1][tid] = d1;
      s_d[2][tid] = d2;
      __syncthreads();
      if (tid == 0)
        for (int k = 0; k < UNWRAP_NT && c0 + k < mb.y; ++k) {
          const R4<R> up = ld4_rw(upos, s_p[k]);
          R4<R> u = ld4_rw(upos, c0 + k);
          u.x = static_cast<R>(static_cast<double>(up.x) + s_d[0][k]);
          u.y = static_cast<R>(static_cast<double>(up.y) + s_d[1][k]);
          u.z = static_cast<R>(static_cast<double>(up.z) + s_d[2][k]);
          st4(upos, c0 + k, u);
        }
      __syncthreads();
      if (active) uy = static_cast<double>(ld4_rw(upos, i).y);
    } else {
      // segment heads take their placed partner's image; a segmented scan
      // over the block adds the bond vectors down each segment
      double a0 = d0, a1 = d1, a2 = d2;
      if (active && !chained) {
        const R4<R> up = ld4_rw(upos, p);
        a0 += static_cast<double>(up.x);
        a1 += static_cast<double>(up.y);
        a2 += static_cast<double>(up.z);
      }
      int head = chained ? -1 : lane;  // inactive lanes head themselves
      for (int o = 1; o < 32; o <<= 1) {
        const int h = __shfl_up_sync(FULL, head, o);
        if (lane >= o && h > head) head = h;
      }
      for (int o = 1; o < 32; o <<= 1) {
        const double t0 = __shfl_up_sync(FULL, a0, o), t1 = __shfl_up_sync(FULL, a1, o),
                     t2 = __shfl_up_sync(FULL, a2, o);
        if (lane >= o && lane - o >= head) {  // head < 0: the segment began before the warp
          a0 += t0;
          a1 += t1;
          a2 += t2;
        }
      }
      if (lane == 31) {
        s_wsum[0][w] = a0;
        s_wsum[1][w] = a1;
        s_wsum[2][w] = a2;
        s_whead[w] = head >= 0;
      }
      __syncthreads();
      if (tid == 0) {  // carry into each warp's leading lanes, warps in order
        double c[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < NW; ++q) {
          for (int k = 0; k < 3; ++k) s_carry[k][q] = c[k];
          for (int k = 0; k < 3; ++k) c[k] = s_whead[q] ? s_wsum[k][q] : c[k] + s_wsum[k][q];
        }
      }
      __syncthreads();
      if (head < 0) {  // this lane's segment began in an earlier warp
        a0 += s_carry[0][w];
        a1 += s_carry[1][w];
        a2 += s_carry[2][w];
      }
      if (active) {
        R4<R> u = ld4_rw(upos, i);
        u.x = static_cast<R>(a0);
        u.y = static_cast<R>(a1);
        u.z = static_cast<R>(a2);
        st4(upos, i, u);
        uy = static_cast<double>(u.y);
      }
    }
    if (active) {  // the image's shear velocity
      const double ny = round((uy - xy) * invL[1]);
      R4<R> v = ld4_rw(uvel, i);
      v.x = static_cast<R>(static_cast<double>(v.x) + ny * sLy);
      st4(uvel, i, v);
    }
    __syncthreads();  // this chunk's images are placed before the next chunk reads them
  }
}

template <typename R>
__global__ void k_profile_centre(const int2* rep_mols, const int2* mols, const R* mpos,
                                 const R* mvel, int rep, double* c6) {
  const int2 rm = rep_mols[rep];
  if (rm.y == 0) {
    for (int k = 0; k < 6; ++k) c6[k] = 0.0;
    return;
  }
  const int2 mb = mols[rm.x];
  molecule_centre<R>(mpos, mvel, mb.x, mb.y, c6);
}

// bins: x then y, 3 doubles per bin (sum v_x, sum v_y, count), zeroed by the host
template <typename R>
__global__ void k_velocity_profile(const RepInfo* reps, int rep, const R* rec, double delrx,
                                   double width, long long kx0, int nx, long long ky0, int ny,
                                   const double* c6, double* bins) {
  const RepInfo& ri = reps[rep];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ri.slot_cap) return;
  const size_t s = static_cast<size_t>(ri.slot_base) + i;
  const R* p = rec + 8 * s;
  if (slot_id(p[3]) == SLOT_EMPTY) return;
  double x0 = static_cast<double>(p[0]) - c6[0], x1 = static_cast<double>(p[1]) - c6[1],
         x2 = static_cast<double>(p[2]) - c6[2];
  double v0 = static_cast<double>(p[4]) - c6[3], v1 = static_cast<double>(p[5]) - c6[4];
  const double Lx = ri.L[0], Ly = ri.L[1], Lz = ri.L[2];
  if (ri.shear != 0.0) {  // MPC::LEBC(pos, vel) (MPC.cpp:431-439)
    const double cy = round(x1 / Ly);
    x0 -= Lx * round(x0 / Lx);
    x0 -= cy * delrx;
    x0 -= Lx * round(x0 / Lx);
    x1 -= Ly * cy;
    x2 -= Lz * round(x2 / Lz);
    v0 -= cy * ri.shear * Ly;
  } else {  // MPC::wrap(pos) (MPC.cpp:473-478)
    x0 -= round(x0 / Lx) * Lx;
    x1 -= round(x1 / Ly) * Ly;
  }
  const long long kx = static_cast<long long>(floor(x0 / width)) - kx0;
  const long long ky = static_cast<long long>(floor(x1 / width)) - ky0;
  if (kx >= 0 && kx < nx) {
    atomicAdd(bins + 3 * kx, v0);
    atomicAdd(bins + 3 * kx + 1, v1);
    atomicAdd(bins + 3 * kx + 2, 1.0);
  }
  if (ky >= 0 && ky < ny) {
    double* b = bins + 3 * static_cast<size_t>(nx);
    atomicAdd(b + 3 * ky, v0);
    atomicAdd(b + 3 * ky + 1, v1);
    atomicAdd(b + 3 * ky + 2, 1.0);
  }
}

}  // namespace smpc
