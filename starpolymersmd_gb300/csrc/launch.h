// Host-side launch entry points for the kernels, instantiated once per
// precision (kernels_fp64.cu compiled with -fmad=false for reference parity,
// kernels_fp32.cu for the fast path).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "smpc_device.cuh"

namespace smpc {

struct MdArgs;
struct PmdArgs;

// Launch-shape variants of the FP32 fast-path kernels, chosen by the
// autotuner (smpc_autotune). The FP64 parity kernels have one shape.
int bin_variant_count();
int collide_variant_count();
int md_variant_count();
int collide_variant_cells(int v);     // cells per collide tile of variant v
const char* bin_variant_name(int v);
const char* collide_variant_name(int v);
const char* md_variant_name(int v);
// periodic-MD shapes: lanes per bead of k_pmd_forces, blocks per SM of the
// list builder k_pmd_nlist (FP32; FP64 keeps one lane per bead)
int pmd_variant_count();
int pmd_variant_lanes(int v);
int pmd_variant_list_blocks_per_sm(int v);
const char* pmd_variant_name(int v);

template <typename R>
struct CollideArgs {
  int variant;
  const FrameF* frames;  // float frames (FP32 path)
  const Tile* tiles;
  int n_tiles;
  const RepInfo* reps;
  const RepDyn* dyn;
  const uint32_t* off;
  const uint32_t* perm;
  const R* st_in;   // solvent slot records (position, velocity)
  R* st_out;
  const R* mpos;
  R* mvel;
  const uint2* mkey;
  const int* mimg;
  const double* inj_gamma;
  const double* inj_uphi;
  const double* inj_utheta;
  int rng;
  double rot_c;
  double rot_s;
  int strict;
  int mono_bin;
  int amc;  // angular-momentum-conserving collision (generic kernel only)
  ErrorState* err;
  // collision-frame records written by the binning just before (generic
  // kernel; FP64 contexts), or null: the collide recomputes them from st_in
  const R* frame;
};

// Tile geometry chosen per precision (register budget of k_collide).
template <typename R>
int collide_cells_per_tile();
int fluid_slots_per_tile(bool fp64);
int temperature_cells_per_tile();
int md_max_monomers();

template <typename R>
void launch_cycle_begin(const RepInfo* reps, RepDyn* dyn, int n_rep, int n_adv, double adv_scale,
                        int gen_shift, cudaStream_t st);
template <typename R>
void launch_cycle_end(RepDyn* dyn, int n_rep, cudaStream_t st);
template <typename R>
void launch_init_solvent(const RepInfo* reps, int rep, int slot_cap, R* rec,
                         unsigned long long seed, double kT, int flags, double* part,
                         cudaStream_t st);
constexpr int INIT_PART_DOUBLES = 3 * 256;  // k_init_velocity_sum partials (INIT_SUM_BLOCKS)
template <typename R>
void launch_mono_prep(const RepInfo* reps, RepDyn* dyn, int n_rep, R* mpos, R* mvel, uint2* mkey,
                      int* mimg, uint32_t* count, ErrorState* err, int mono_bin, int strict,
                      FrameF* frames, double rot_c, double rot_s, int chunks, cudaStream_t st);
template <typename R>
void launch_fluid_bin(const Tile* tiles, int n_tiles, const RepInfo* reps, const RepDyn* dyn,
                      const FrameF* frames, const R* rec, uint2* keys, uint32_t* count,
                      ErrorState* err, int strict, int variant, int packed, R* frame,
                      cudaStream_t st);
template <typename R>
void launch_collide(const CollideArgs<R>& a, cudaStream_t st);
template <typename R>
void launch_temperature(const Tile* tiles, int n_tiles, const RepInfo* reps, const uint32_t* off,
                        const uint32_t* perm, const R* rec_cur, const R* mpos, const R* mvel,
                        const int* mimg, int mono_bin, TempPartial* partial, cudaStream_t st);
// A second stream with fork / join events for the MD launch shape that runs
// two kernels side by side (variant 3): replicas order[0, n_big) of the MD
// order (more than 512 monomers) on 1024-thread blocks, the rest on
// 512-thread blocks, two of which fit one SM.
struct MdSplit {
  cudaStream_t st2;
  cudaEvent_t fork, join;
  int n_big;
  int cluster;  // > 0: non-periodic MD on clusters of this many CTAs per replica (k_md_cluster)
};
// Largest cluster size (16 or 8) at which k_md_cluster<R> can run on the
// current device (0: none); enables the non-portable size 16 on the kernel.
template <typename R>
int md_cluster_size();
constexpr int MD_CLUSTER_CAP_HOST = 1024;  // beads per replica k_md_cluster holds (MD_CLUSTER_CAP)
template <typename R>
void launch_md(const MdArgs& a, int n_rep, R* mpos, R* mvel, R* mfrc, R* mver, int variant,
               cudaStream_t st, const MdSplit& split);

// n MD substeps of one periodic box (pmd_kernels.cuh); n = 0 builds lists
// and forces only (set-up). mnext: second position buffer of the box.
template <typename R>
void launch_pmd_call(const PmdArgs& a, const RepInfo* reps, RepDyn* dyn, R* mpos, R* mnext,
                     R* mvel, R* mfrc, R* mdisp, int n, double adv_scale, int calc_epot,
                     int variant, cudaStream_t st);
int pmd_block_count(int n_beads);

// Molecules of periodic boxes made whole (observables.cuh); other boxes copied.
template <typename R>
void launch_unwrap_molecules(const RepInfo* reps, const RepDyn* dyn, const int2* mols,
                             const int* mol_rep, int n_mols, int n_mono, const int* bond_start,
                             const int2* bonds, const R* mpos, const R* mvel, R* upos, R* uvel,
                             cudaStream_t st);

// Output-step observables: per molecule into mol_out (OBS_PER_REP each), then
// per replica into out.
template <typename R>
void launch_mol_observables(const int2* rep_mols, const int2* mols, int n_rep, int n_mols,
                            const R* mpos, const R* mvel, double* mol_out, double* out,
                            cudaStream_t st);
template <typename R>
void launch_velocity_profile(const RepInfo* reps, const int2* rep_mols, const int2* mols, int rep,
                             int slot_cap, const R* rec, const R* mpos, const R* mvel,
                             double delrx, double width, long long kx0, int nx, long long ky0,
                             int ny, double* c6, double* bins, cudaStream_t st);

// Solvent analyses (analysis.cuh); part: per-block partial sums.
template <typename R>
void launch_fourier_modes(const RepInfo* reps, int rep, const R* rec, double kwave, double* part,
                          int n_blocks, cudaStream_t st);
template <typename R>
void launch_vacf_sample(const RepInfo* reps, int rep, int slot_cap, const R* rec, int n_p,
                        int slot, double* ring, cudaStream_t st);
template <typename R>
void launch_vacf_lags(const double* ring, int n_p, int entries, int first, double* part,
                      int n_blocks, cudaStream_t st);

// Pressure tensor parts (analysis.cuh): solvent kinetic per slot tile
// (part[6 * tile]), monomer kinetic + virial per replica (out[12 * r]).
template <typename R>
void launch_kinetic_tensor(const Tile* tiles, int n_tiles, const RepInfo* reps, const R* rec,
                           double* part, cudaStream_t st);
template <typename R>
void launch_mono_stress(const RepInfo* reps, const RepDyn* dyn, int n_rep, const R* mpos,
                        const R* mvel, const int* nlist_t, const int* ncount, int n_mono_total,
                        int* const* rows, int max_nb, const int* bond_start, const int2* bonds,
                        double* out, cudaStream_t st);

// Monomer state between the C ABI's x,y,z-interleaved doubles and the device
// records (pos.w / vel.w keep mass and type): pos, vel, frc each 3M doubles, in
// the device staging buffer or in pinned host memory the device maps
template <typename R>
void launch_unpack_monomers(const double* pos, const double* vel, int n, R* mpos, R* mvel,
                            cudaStream_t st);
template <typename R>
void launch_pack_monomers(const R* mpos, const R* mvel, const R* mfrc, int n, double* pos,
                          double* vel, double* frc, cudaStream_t st);

void launch_scan(uint32_t* count, uint32_t* off, uint32_t* tile_sum, uint32_t* grand, int n_cells,
                 cudaStream_t st);
int scan_tile_count(int n_cells);
void launch_build_perm(const uint2* keys, int n_slots, const uint2* mkey, int n_mono,
                       const uint32_t* off, uint32_t* perm, ErrorState* err, cudaStream_t st);
// the same from packed solvent keys (local cell << 16 | rank), one block per
// binning tile of slots
void launch_build_perm_packed(const Tile* tiles, int n_tiles, const RepInfo* reps,
                              const uint32_t* keys, int n_slots, const uint2* mkey, int n_mono,
                              const uint32_t* off, uint32_t* perm, ErrorState* err,
                              cudaStream_t st);

}  // namespace smpc
