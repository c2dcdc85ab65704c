// Launch wrappers shared by kernels_fp64.cu and kernels_fp32.cu; each of
// those defines SMPC_REAL and the tile constants and includes this file once.
#pragma once
#include <algorithm>
#include "launch.h"
#include "md_kernels.cuh"
#include "mpc_fast.cuh"
#include "mpc_kernels.cuh"
#include "observables.cuh"
#include "pmd_kernels.cuh"
#include "analysis.cuh"

namespace smpc {

typedef SMPC_REAL Real;

template <>
int collide_cells_per_tile<Real>() {
  return SMPC_COLLIDE_CT;
}

template <>
void launch_cycle_begin<Real>(const RepInfo* reps, RepDyn* dyn, int n_rep, int n_adv,
                              double adv_scale, int gen_shift, cudaStream_t st) {
  k_cycle_begin<Real><<<(n_rep + 127) / 128, 128, 0, st>>>(reps, dyn, n_rep, n_adv, adv_scale,
                                                           gen_shift);
}

template <>
void launch_cycle_end<Real>(RepDyn* dyn, int n_rep, cudaStream_t st) {
  k_cycle_end<Real><<<(n_rep + 127) / 128, 128, 0, st>>>(dyn, n_rep);
}

template <>
void launch_init_solvent<Real>(const RepInfo* reps, int rep, int slot_cap, Real* rec,
                               unsigned long long seed, double kT, int flags, double* part,
                               cudaStream_t st) {
  static_assert(INIT_PART_DOUBLES == 3 * INIT_SUM_BLOCKS, "partials buffer size");
  if (slot_cap == 0) return;
  k_init_solvent<Real><<<(slot_cap + 255) / 256, 256, 0, st>>>(reps, rep, rec, seed, kT, flags);
  k_init_velocity_sum<Real><<<INIT_SUM_BLOCKS, INIT_SUM_THREADS, 0, st>>>(reps, rep, rec, part);
  k_init_velocity_finish<Real><<<INIT_SUM_BLOCKS, 256, 0, st>>>(reps, rep, rec, part, flags);
}

template <>
void launch_mono_prep<Real>(const RepInfo* reps, RepDyn* dyn, int n_rep, Real* mpos, Real* mvel,
                            uint2* mkey, int* mimg, uint32_t* count, ErrorState* err,
                            int mono_bin, int strict, FrameF* frames, double rot_c, double rot_s,
                            int chunks, cudaStream_t st) {
  const dim3 grid(n_rep, chunks > 0 ? chunks : 1);
  k_mono_prep<Real, 256><<<grid, 256, 0, st>>>(reps, dyn, mpos, mvel, mkey, mimg, count, err,
                                               mono_bin, strict, frames, rot_c, rot_s);
}

#if SMPC_FAST_F32
template <int NT, int U>
void bin_f32(const Tile* tiles, int n_tiles, const RepInfo* reps, const FrameF* frames,
             const float* rec, uint2* keys, uint32_t* count, ErrorState* err, bool packed,
             cudaStream_t st) {
  if (packed)
    k_fluid_bin_f32<NT, U, true><<<n_tiles, NT, 0, st>>>(tiles, reps, frames, rec, keys, count, err);
  else
    k_fluid_bin_f32<NT, U, false><<<n_tiles, NT, 0, st>>>(tiles, reps, frames, rec, keys, count,
                                                          err);
}

template <int NT, int CT, int CAP, int GU>
void collide_f32(const CollideArgs<float>& a, cudaStream_t st) {
  auto kern = k_collide_f32<NT, CT, CAP, GU>;
  const size_t dyn = collide_f32_dyn_smem(CAP);
  static bool configured = false;  // the attribute is per function, set once
  if (!configured) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dyn));
    configured = true;
  }
  kern<<<a.n_tiles, NT, dyn, st>>>(a.tiles, a.reps, a.frames, a.dyn, a.off, a.perm, a.st_in,
                                   a.st_out, a.mpos, a.mvel, a.mimg, a.inj_gamma, a.inj_uphi,
                                   a.inj_utheta, a.rng, a.mono_bin, a.err);
}

template <int NT, int CT, int CAP>
void collide_f32_async(const CollideArgs<float>& a, cudaStream_t st) {
  auto kern = k_collide_f32_async<NT, CT, CAP>;
  const size_t dyn = collide_f32_dyn_smem(CAP);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dyn));
    configured = true;
  }
  kern<<<a.n_tiles, NT, dyn, st>>>(a.tiles, a.reps, a.frames, a.dyn, a.off, a.perm, a.st_in,
                                   a.st_out, a.mpos, a.mvel, a.mimg, a.inj_gamma, a.inj_uphi,
                                   a.inj_utheta, a.rng, a.mono_bin, a.err);
}
#endif

template <>
void launch_fluid_bin<Real>(const Tile* tiles, int n_tiles, const RepInfo* reps,
                            const RepDyn* dyn, const FrameF* frames, const Real* rec, uint2* keys,
                            uint32_t* count, ErrorState* err, int strict, int variant,
                            int packed, Real* frame, cudaStream_t st) {
  if (n_tiles == 0) return;
#if SMPC_FAST_F32
  if (!strict && variant >= 0) {  // variant < 0: the generic kernel (what k_collide recomputes)
    const bool pk = packed != 0;
    switch (variant) {
      case 1: bin_f32<256, 2>(tiles, n_tiles, reps, frames, rec, keys, count, err, pk, st); return;
      case 2: bin_f32<256, 8>(tiles, n_tiles, reps, frames, rec, keys, count, err, pk, st); return;
      case 3: bin_f32<128, 8>(tiles, n_tiles, reps, frames, rec, keys, count, err, pk, st); return;
      default: bin_f32<256, 4>(tiles, n_tiles, reps, frames, rec, keys, count, err, pk, st); return;
    }
  }
#else
  (void)packed;
#endif
  (void)frames;
  (void)variant;
  k_fluid_bin<Real, SMPC_BIN_NT><<<n_tiles, SMPC_BIN_NT, 0, st>>>(tiles, reps, dyn, rec, keys,
                                                                  count, err, strict, frame);
}

template <>
void launch_collide<Real>(const CollideArgs<Real>& a, cudaStream_t st) {
  if (a.n_tiles == 0) return;
#if SMPC_FAST_F32
  if (!a.strict && !a.amc) {
    switch (a.variant) {
      case 1: collide_f32<256, 128, 1408, 8>(a, st); return;
      case 2: collide_f32<128, 64, 704, 4>(a, st); return;
      case 3: collide_f32<128, 64, 704, 8>(a, st); return;
      case 4: collide_f32<512, 256, 2816, 4>(a, st); return;
      case 5: collide_f32_async<128, 64, 704>(a, st); return;
      case 6: collide_f32_async<256, 128, 1408>(a, st); return;
      case 7: collide_f32_async<128, 64, 736>(a, st); return;
      case 8: collide_f32_async<128, 64, 768>(a, st); return;
      case 9: collide_f32_async<160, 64, 704>(a, st); return;
      case 10: collide_f32_async<192, 64, 704>(a, st); return;
      case 11: collide_f32_async<256, 64, 704>(a, st); return;
      default: collide_f32<256, 128, 1408, 4>(a, st); return;
    }
  }
#endif
  auto kern = k_collide<Real, SMPC_COLLIDE_NT, SMPC_COLLIDE_CT, SMPC_COLLIDE_CAP>;
  const size_t dyn = collide_dyn_smem<Real>(SMPC_COLLIDE_CAP);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dyn));
    configured = true;
  }
  kern<<<a.n_tiles, SMPC_COLLIDE_NT, dyn, st>>>(
      a.tiles, a.reps, a.dyn, a.off, a.perm, a.st_in, a.st_out, a.mpos, a.mvel, a.mkey, a.mimg,
      a.inj_gamma, a.inj_uphi, a.inj_utheta, a.rng, a.rot_c, a.rot_s, a.strict, a.mono_bin, a.amc,
      a.err, a.frame);
}

template <>
void launch_temperature<Real>(const Tile* tiles, int n_tiles, const RepInfo* reps,
                              const uint32_t* off, const uint32_t* perm, const Real* rec_cur,
                              const Real* mpos, const Real* mvel, const int* mimg, int mono_bin,
                              TempPartial* partial, cudaStream_t st) {
  if (n_tiles == 0) return;
  k_temperature<Real, 128><<<n_tiles, 128, 0, st>>>(tiles, reps, off, perm, rec_cur, mpos, mvel,
                                                    mimg, mono_bin, partial);
}

template <>
void launch_mol_observables<Real>(const int2* rep_mols, const int2* mols, int n_rep, int n_mols,
                                  const Real* mpos, const Real* mvel, double* mol_out,
                                  double* out, cudaStream_t st) {
  if (n_rep == 0) return;
  if (n_mols > 0) k_mol_observables<Real, 256><<<n_mols, 256, 0, st>>>(mols, mpos, mvel, mol_out);
  k_obs_reduce<Real><<<(n_rep + 3) / 4, 128, 0, st>>>(rep_mols, mol_out, n_rep, out);
}

template <>
void launch_unwrap_molecules<Real>(const RepInfo* reps, const RepDyn* dyn, const int2* mols,
                                   const int* mol_rep, int n_mols, int n_mono,
                                   const int* bond_start, const int2* bonds, const Real* mpos,
                                   const Real* mvel, Real* upos, Real* uvel, cudaStream_t st) {
  if (n_mono == 0) return;
  k_copy_monomers<Real><<<std::min((n_mono + 255) / 256, 152 * 8), 256, 0, st>>>(n_mono, mpos, mvel,
                                                                              upos, uvel);
  if (n_mols > 0)
    k_unwrap_molecules<Real><<<n_mols, UNWRAP_NT, 0, st>>>(reps, dyn, mols, mol_rep, n_mols,
                                                           bond_start, bonds, mpos, mvel, upos,
                                                           uvel);
}

template <>
void launch_fourier_modes<Real>(const RepInfo* reps, int rep, const Real* rec, double kwave,
                                double* part, int n_blocks, cudaStream_t st) {
  k_fourier_modes<Real><<<n_blocks, ANA_NT, 0, st>>>(reps, rep, rec, kwave, part);
}

template <>
void launch_vacf_sample<Real>(const RepInfo* reps, int rep, int slot_cap, const Real* rec,
                              int n_p, int slot, double* ring, cudaStream_t st) {
  if (slot_cap == 0) return;
  k_vacf_sample<Real><<<std::min((slot_cap + ANA_NT - 1) / ANA_NT, 152 * 8), ANA_NT, 0, st>>>(
      reps, rep, rec, n_p, slot, ring);
}

template <>
void launch_vacf_lags<Real>(const double* ring, int n_p, int entries, int first, double* part,
                            int n_blocks, cudaStream_t st) {
  k_vacf_lags<Real><<<dim3(n_blocks, entries), ANA_NT, 0, st>>>(ring, n_p, entries, first, part);
}

template <>
void launch_kinetic_tensor<Real>(const Tile* tiles, int n_tiles, const RepInfo* reps,
                                 const Real* rec, double* part, cudaStream_t st) {
  if (n_tiles == 0) return;
  k_kinetic_tensor<Real><<<n_tiles, ANA_NT, 0, st>>>(tiles, reps, rec, part);
}

template <>
void launch_mono_stress<Real>(const RepInfo* reps, const RepDyn* dyn, int n_rep, const Real* mpos,
                              const Real* mvel, const int* nlist_t, const int* ncount,
                              int n_mono_total, int* const* rows, int max_nb,
                              const int* bond_start, const int2* bonds, double* out,
                              cudaStream_t st) {
  if (n_rep == 0) return;
  k_mono_stress<Real><<<n_rep, ANA_NT, 0, st>>>(reps, dyn, mpos, mvel, nlist_t, ncount,
                                                n_mono_total, rows, max_nb, bond_start, bonds,
                                                out);
}

template <>
void launch_pmd_call<Real>(const PmdArgs& a, const RepInfo* reps, RepDyn* dyn, Real* mpos,
                           Real* mnext, Real* mvel, Real* mfrc, Real* mdisp, int n,
                           double adv_scale, int calc_epot, int variant, cudaStream_t st) {
  if (a.n == 0) return;
  const int nb = a.n_blocks;
#if SMPC_FAST_F32
  const int lanes = pmd_variant_lanes(variant);
  const int list_bps = pmd_variant_list_blocks_per_sm(variant);
#else
  (void)variant;
  const int lanes = pmd_force_lanes<Real>();
  const int list_bps = 4;
#endif
  // k_pmd_nlist: warps stride over the beads, list_bps blocks per SM of GB300
  // (a launch without a rebuild request returns at once and stays short)
  const int nb_list = std::min((a.n + PMD_NT / 32 - 1) / (PMD_NT / 32), 152 * list_bps);
  const int nb_force = pmd_force_block_count(a.n, lanes);
  auto forces = k_pmd_forces<Real, pmd_force_lanes<Real>()>;
#if SMPC_FAST_F32
  if (lanes == 4) forces = k_pmd_forces<Real, 4>;
  if (lanes == 16) forces = k_pmd_forces<Real, 16>;
#endif
  if (n == 0) {
    k_pmd_drift<Real><<<nb, PMD_NT, 0, st>>>(a, reps, dyn, mpos, mvel, mfrc, mdisp, 0, adv_scale, 0);
    k_pmd_nlist<Real><<<nb_list, PMD_NT, 0, st>>>(a, reps, mpos, mdisp, 0, adv_scale);
    forces<<<nb_force, PMD_NT, 0, st>>>(a, reps, dyn, mpos, mnext, mvel, mfrc, mdisp, 0, adv_scale,
                                        0, 0, calc_epot);
    return;
  }
  k_pmd_drift<Real><<<nb, PMD_NT, 0, st>>>(a, reps, dyn, mpos, mvel, mfrc, mdisp, 1, adv_scale, 1);
  // the kernels after the drift follow their predecessor programmatically
  // (pmd_wait_previous): their launch overlaps its last blocks
  cudaLaunchAttribute pdl[1];
  pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  pdl[0].val.programmaticStreamSerializationAllowed = 1;
  auto cfg = [&](int blocks) {
    cudaLaunchConfig_t c = {};
    c.gridDim = dim3(blocks);
    c.blockDim = dim3(PMD_NT);
    c.dynamicSmemBytes = 0;
    c.stream = st;
    c.attrs = pdl;
    c.numAttrs = 1;
    return c;
  };
  for (int k = 1; k <= n; ++k) {
    Real* pin = (k & 1) ? mpos : mnext;  // substep k's positions: buffer (k - 1) & 1
    Real* pout = (k & 1) ? mnext : mpos;
    const cudaLaunchConfig_t cl = cfg(nb_list);
    cudaLaunchKernelEx(&cl, k_pmd_nlist<Real>, a, reps, static_cast<const Real*>(pin), mdisp, k,
                       adv_scale);
    const cudaLaunchConfig_t cf = cfg(nb_force);
    cudaLaunchKernelEx(&cf, forces, a, reps, dyn, static_cast<const Real*>(pin), pout,
                       mvel, mfrc, mdisp, k, adv_scale, 1, static_cast<int>(k < n),
                       static_cast<int>(calc_epot && k == n));
  }
  if ((n & 1) == 0) {
    const cudaLaunchConfig_t cc = cfg(nb);
    cudaLaunchKernelEx(&cc, k_pmd_copy<Real>, a, static_cast<const Real*>(mnext), mpos);
  }
}

template <>
void launch_velocity_profile<Real>(const RepInfo* reps, const int2* rep_mols, const int2* mols,
                                   int rep, int slot_cap, const Real* rec, const Real* mpos,
                                   const Real* mvel, double delrx, double width, long long kx0,
                                   int nx, long long ky0, int ny, double* c6, double* bins,
                                   cudaStream_t st) {
  k_profile_centre<Real><<<1, 1, 0, st>>>(rep_mols, mols, mpos, mvel, rep, c6);
  if (slot_cap == 0) return;
  k_velocity_profile<Real><<<(slot_cap + 255) / 256, 256, 0, st>>>(
      reps, rep, rec, delrx, width, kx0, nx, ky0, ny, c6, bins);
}

// Monomer state between the device's R4 records and x,y,z-interleaved double
// arrays: a device staging buffer, or the caller's pinned host arrays read and
// written in place over the C2C link (the host pointer is the device pointer).
template <typename R>
__global__ void k_unpack_monomers(const double* __restrict__ pos, const double* __restrict__ vel,
                                  int n, R* mpos, R* mvel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = pos + 3 * static_cast<size_t>(i);
  const double* v = vel + 3 * static_cast<size_t>(i);
  R4<R> x = ld4_rw(mpos, i), u = ld4_rw(mvel, i);
  x.x = static_cast<R>(p[0]);
  x.y = static_cast<R>(p[1]);
  x.z = static_cast<R>(p[2]);
  u.x = static_cast<R>(v[0]);
  u.y = static_cast<R>(v[1]);
  u.z = static_cast<R>(v[2]);
  st4(mpos, i, x);
  st4(mvel, i, u);
}

template <typename R>
__global__ void k_pack_monomers(const R* mpos, const R* mvel, const R* mfrc, int n,
                                double* __restrict__ pos, double* __restrict__ vel,
                                double* __restrict__ frc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const R4<R> x = ld4_rw(mpos, i), u = ld4_rw(mvel, i);
  double* p = pos + 3 * static_cast<size_t>(i);
  double* v = vel + 3 * static_cast<size_t>(i);
  p[0] = static_cast<double>(x.x);
  p[1] = static_cast<double>(x.y);
  p[2] = static_cast<double>(x.z);
  v[0] = static_cast<double>(u.x);
  v[1] = static_cast<double>(u.y);
  v[2] = static_cast<double>(u.z);
  if (mfrc && frc) {
    const R4<R> fr = ld4_rw(mfrc, i);
    double* q = frc + 3 * static_cast<size_t>(i);
    q[0] = static_cast<double>(fr.x);
    q[1] = static_cast<double>(fr.y);
    q[2] = static_cast<double>(fr.z);
  }
}

template <>
void launch_unpack_monomers<Real>(const double* pos, const double* vel, int n, Real* mpos,
                                  Real* mvel, cudaStream_t st) {
  if (n > 0) k_unpack_monomers<Real><<<(n + 255) / 256, 256, 0, st>>>(pos, vel, n, mpos, mvel);
}

template <>
void launch_pack_monomers<Real>(const Real* mpos, const Real* mvel, const Real* mfrc, int n,
                                double* pos, double* vel, double* frc, cudaStream_t st) {
  if (n > 0)
    k_pack_monomers<Real><<<(n + 255) / 256, 256, 0, st>>>(mpos, mvel, mfrc, n, pos, vel, frc);
}

// dynamic shared memory of k_md_cluster (the compacted force pass), opted in
// once per cluster size
template <int CS>
static size_t md_cluster_smem() {
  constexpr size_t bytes = MdcLayout<Real, CS>::bytes;
  static const bool set = cudaFuncSetAttribute(k_md_cluster<Real, 256, CS, 8>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(bytes)) == cudaSuccess;
  (void)set;
  return bytes;
}

template <int CS>
static cudaError_t launch_md_cluster_cs(const MdArgs& a, int n_rep, Real* mpos, Real* mvel,
                                        Real* mfrc, Real* mver, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(n_rep * CS));
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = md_cluster_smem<CS>();
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MdArgs b = a;
  b.order = nullptr;
  return cudaLaunchKernelEx(&cfg, k_md_cluster<Real, 256, CS, 8>, b, mpos, mvel, mfrc, mver);
}

template <int CS>
static int cluster_fits() {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CS);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = md_cluster_smem<CS>();
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_md_cluster<Real, 256, CS, 8>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <>
int md_cluster_size<Real>() {
  if (cudaFuncSetAttribute(k_md_cluster<Real, 256, 16, 8>,
                           cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
      cluster_fits<16>() > 0)
    return 16;
  cudaGetLastError();
  return cluster_fits<8>() > 0 ? 8 : 0;
}

template <>
void launch_md<Real>(const MdArgs& a, int n_rep, Real* mpos, Real* mvel, Real* mfrc, Real* mver,
                     int variant, cudaStream_t st, const MdSplit& split) {
  if (n_rep == 0) return;
  static_assert(MD_CLUSTER_CAP == MD_CLUSTER_CAP_HOST, "cluster MD capacity");
  // FP64: whenever the context chose clusters, unless variant 1 asks for one
  // CTA per replica; FP32: launch-shape variant 4
  if (split.cluster > 0 && !a.lowe && (SMPC_FAST_F32 ? variant == 4 : variant != 1)) {
    if (split.cluster == 16)
      launch_md_cluster_cs<16>(a, n_rep, mpos, mvel, mfrc, mver, st);
    else
      launch_md_cluster_cs<8>(a, n_rep, mpos, mvel, mfrc, mver, st);
    return;
  }
  MdArgs b = a;
#if SMPC_FAST_F32
  if (variant == 3 && split.n_big > 0 && split.n_big < n_rep && a.order) {
    // big replicas on the forked stream, small ones here; joined before return
    cudaEventRecord(split.fork, st);
    cudaStreamWaitEvent(split.st2, split.fork, 0);
    k_md_substeps<Real, 1024, 1, 8><<<split.n_big, 1024, 0, split.st2>>>(b, mpos, mvel, mfrc, mver);
    MdArgs c = a;
    c.order = a.order + split.n_big;
    k_md_substeps<Real, 512, 1, 8><<<n_rep - split.n_big, 512, 0, st>>>(c, mpos, mvel, mfrc, mver);
    cudaEventRecord(split.join, split.st2);
    cudaStreamWaitEvent(st, split.join, 0);
    return;
  }
  if (variant == 2 || variant == 3) {
    k_md_substeps<Real, 1024, 1, 8><<<n_rep, 1024, 0, st>>>(b, mpos, mvel, mfrc, mver);
    return;
  }
  b.order = nullptr;
  if (variant == 1) {
    k_md_substeps<Real, 512, 2><<<n_rep, 512, 0, st>>>(b, mpos, mvel, mfrc, mver);
    return;
  }
#endif
  (void)variant;
  b.order = nullptr;
  k_md_substeps<Real, SMPC_MD_NT, SMPC_MD_MPT><<<n_rep, SMPC_MD_NT, 0, st>>>(b, mpos, mvel, mfrc,
                                                                          mver);
}

}  // namespace smpc
