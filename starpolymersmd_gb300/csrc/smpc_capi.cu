// C-ABI implementation (include/smpc.h): device context, uploads/downloads,
// the step-by-step reference-compatible calls and the graph-captured fused
// cycle. All device memory is allocated at creation (and when bonds are
// uploaded); the step calls allocate nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <new>
#include <vector>

#include "../../include/smpc.h"
#include "launch.h"
#include "md_kernels.cuh"
#include "observables.cuh"
#include "pmd_kernels.cuh"
#include "smpc_device.cuh"

using smpc::ErrorState;
using smpc::RepDyn;
using smpc::RepInfo;
using smpc::TempPartial;
using smpc::Tile;

struct smpc_ctx {
  smpc_options opt{};
  int n_rep = 0;
  std::vector<RepInfo> reps;
  std::vector<RepDyn> dyn;  // host mirror: delrx, shift, h are host-owned in step mode
  std::vector<int> n_fluid, mol0;
  long long total_cells = 0, total_slots = 0, total_mono = 0;
  cudaStream_t st = nullptr;
  int device = 0;
  size_t real_size = 8;

  RepInfo* d_reps = nullptr;
  RepDyn* d_dyn = nullptr;
  Tile* d_bin_tiles = nullptr;
  int n_bin_tiles = 0;
  std::vector<int> bin_tile_rep;  // replica of each binning tile
  Tile* d_col_tiles = nullptr;   // parity-path collide tiles
  int n_col_tiles = 0;
  // fast path: collide tiles for each tile size the variants use (64/128/256 cells)
  Tile* d_col_tiles_v[3] = {nullptr, nullptr, nullptr};
  int n_col_tiles_v[3] = {0, 0, 0};
  int var_bin = 0, var_col = 0, var_md = 0, var_pmd = 0;
  // FP32 fast path, every box at most 65,536 cells: 32-bit sort keys
  bool packed_keys = false;
  std::vector<Tile> h_tmp_tiles;
  Tile* d_tmp_tiles = nullptr;
  TempPartial* d_tpart = nullptr;

  void* d_rec[2] = {nullptr, nullptr};  // solvent slot records: 8 Reals (pos, vel) each
  int cur = 0;
  uint2* d_keys = nullptr;
  uint32_t* d_perm = nullptr;
  uint32_t* d_count = nullptr;
  uint32_t* d_off = nullptr;
  uint32_t* d_tsum = nullptr;
  uint32_t* d_grand = nullptr;

  void* d_mpos = nullptr;
  void* d_mvel = nullptr;
  void* d_mfrc = nullptr;
  void* d_mver = nullptr;
  uint2* d_mkey = nullptr;
  int* d_mimg = nullptr;
  int* d_bond_start = nullptr;
  int2* d_bonds = nullptr;
  int* d_nlist = nullptr;
  int* d_ncount = nullptr;
  int* d_md_order = nullptr;  // replicas by decreasing monomer count (MD CTA order)
  smpc::MdSplit md_split{};   // side-by-side MD launch shape: second stream, events, split
  void* d_lowe = nullptr;     // Lowe-Andersen collision entries, LOWE_MAX per monomer
  RepDyn* h_dyn_pinned = nullptr;  // pinned staging copy of dyn for upload_host_dyn
  cudaEvent_t dyn_ev = nullptr;    // recorded after each staged upload
  bool dyn_ev_pending = false;
  bool any_local_md = false;  // a non-periodic replica has monomers
  // Andersen resets staged for the next smpc_md_substeps (smpc_stage_andersen):
  // per replica the staged substep count (-1: none) and the host tables; the
  // device copy (starts, then monomers) lives in d_and_i / d_and_v while a
  // staged call's MD launch is issued
  std::vector<int> and_steps;
  std::vector<std::vector<int>> and_start_h, and_mono_h;
  std::vector<std::vector<double>> and_vel_h;
  int* d_and_i = nullptr;
  double* d_and_v = nullptr;
  size_t and_i_cap = 0, and_v_cap = 0;
  const int* and_start_dev = nullptr;  // set only while a staged launch is issued
  const int* and_mono_dev = nullptr;
  const double* and_vel_dev = nullptr;
  int mono_chunks = 1;        // CTAs per replica of k_mono_prep (replicas that cannot recentre)
  // periodic boxes (SMPC_REPLICA_PERIODIC_MD): launch arguments with their grid
  // buffers, and molecules made whole for the observables
  std::vector<smpc::PmdArgs> pmd;
  std::vector<void*> pmd_mem;
  void* d_upos = nullptr;
  void* d_uvel = nullptr;
  void* d_mnext = nullptr;    // second monomer position buffer of the periodic MD
  uint8_t* d_pamphi = nullptr;  // solvophobic flag per monomer (periodic MD)
  // solvent analyses: per-block partials, and the velocity-autocorrelation ring
  double* d_ana_part = nullptr;
  size_t ana_part_cap = 0;
  double* d_vacf_ring = nullptr;
  int** d_rows_by_rep = nullptr;  // each replica's periodic Verlet rows, or null
  double* d_stress = nullptr;     // 12 per replica
  int vacf_rep = -1, vacf_np = 0, vacf_entries = 0;
  uint64_t vacf_samples = 0, vacf_calcs = 0;
  std::vector<double> vacf_sum;
  std::vector<std::vector<int>> bsrc, bdst;
  std::vector<std::vector<int>> anchor;

  double* d_inj = nullptr;  // gamma | u_phi | u_theta, total_cells each
  ErrorState* d_err = nullptr;
  smpc::FrameF* d_frames = nullptr;
  // molecules per replica (local monomer offsets) and their device tables
  std::vector<std::vector<int>> mol_start;
  int2* d_rep_mols = nullptr;  // per replica: first molecule, count
  int2* d_mols = nullptr;      // per molecule: global monomer range
  double* d_obs = nullptr;     // OBS_PER_REP per replica
  double* d_mol_obs = nullptr; // OBS_PER_REP per molecule
  int* d_mol_rep = nullptr;    // replica of each molecule
  int n_mols = 0;
  double* d_prof = nullptr;    // velocity-profile bins, grown on demand
  size_t prof_cap = 0;
  double* d_c6 = nullptr;      // centre of molecule 0 (position, velocity)
  double* d_init_part = nullptr;  // solvent initialisation: block sums of the velocities
  double rot_c = 0, rot_s = 0;
  int max_nb = 192;
  bool collided = false;
  bool binned = false;      // smpc_mpc_bin done, collide pending
  // FP64: collision-frame records of the solvent, written by every binning
  // for the collide that follows; frame_ok while the records still match the
  // state (host writes of the solvent clear it)
  void* d_frame = nullptr;
  bool frame_ok = false;
  // per replica: its solvent records sit in the last sort's cell order (set by
  // a collision, cleared by a host upload or a new binning)
  std::vector<uint8_t> sorted;
  bool bin_philox = false;  // that binning drew its shift from Philox
  bool md_ready = false;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  std::string err;
  // host staging reused across calls
  double* d_dstage = nullptr;       // monomer state as the C ABI lays it out (9 x total_mono)
  std::vector<double> h_mass;       // per monomer (pos.w)
  std::vector<double> h_flags;      // amphi + 2*anchor (vel.w)
  std::vector<TempPartial> stage_t;
};

namespace {

bool fast_path(const smpc_ctx* ctx) {
  return ctx->opt.precision == SMPC_FP32 && !ctx->opt.strict_cells && !ctx->opt.angular_momentum;
}
int tile_set(int cells) { return cells == 64 ? 0 : (cells == 128 ? 1 : 2); }

int fail(smpc_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CU(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(ctx, SMPC_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
}

int check_rep(smpc_ctx* ctx, int rep) {
  if (!ctx) return SMPC_E_ARG;
  if (rep < 0 || rep >= ctx->n_rep) return fail(ctx, SMPC_E_ARG, "replica index out of range");
  return SMPC_OK;
}

// Host copy of the RepDyn fields the host owns (delrx, shift[3], h): the
// leading 40 bytes of each record, written with one strided copy.
constexpr size_t kHostDynBytes = offsetof(RepDyn, com);

// The host-owned head of every replica's RepDyn to the device. From a pinned
// staging copy, so the copy is queued without draining the stream first (a
// copy from pageable memory would); the staging copy is rewritten only once
// the previous upload has left it.
int upload_host_dyn(smpc_ctx* ctx) {
  if (!ctx->h_dyn_pinned) {
    CU(cudaMemcpy2DAsync(ctx->d_dyn, sizeof(RepDyn), ctx->dyn.data(), sizeof(RepDyn),
                         kHostDynBytes, ctx->n_rep, cudaMemcpyHostToDevice, ctx->st));
    return SMPC_OK;
  }
  if (ctx->dyn_ev_pending) CU(cudaEventSynchronize(ctx->dyn_ev));
  std::memcpy(ctx->h_dyn_pinned, ctx->dyn.data(), sizeof(RepDyn) * ctx->dyn.size());
  CU(cudaMemcpy2DAsync(ctx->d_dyn, sizeof(RepDyn), ctx->h_dyn_pinned, sizeof(RepDyn),
                       kHostDynBytes, ctx->n_rep, cudaMemcpyHostToDevice, ctx->st));
  CU(cudaEventRecord(ctx->dyn_ev, ctx->st));
  ctx->dyn_ev_pending = true;
  return SMPC_OK;
}

template <typename R>
smpc::CollideArgs<R> collide_args(smpc_ctx* ctx, int rng, int cur);

// the counting sort's scatter, from the keys the binning wrote
void launch_permutation(smpc_ctx* ctx) {
  if (ctx->packed_keys)
    smpc::launch_build_perm_packed(ctx->d_bin_tiles, ctx->n_bin_tiles, ctx->d_reps,
                                   reinterpret_cast<const uint32_t*>(ctx->d_keys),
                                   static_cast<int>(ctx->total_slots), ctx->d_mkey,
                                   static_cast<int>(ctx->total_mono), ctx->d_off, ctx->d_perm,
                                   ctx->d_err, ctx->st);
  else
    smpc::launch_build_perm(ctx->d_keys, static_cast<int>(ctx->total_slots), ctx->d_mkey,
                            static_cast<int>(ctx->total_mono), ctx->d_off, ctx->d_perm, ctx->d_err,
                            ctx->st);
}

template <typename R>
int launch_binning(smpc_ctx* ctx, int cur) {
  const int strict = ctx->opt.strict_cells;
  const R* rec_in = static_cast<const R*>(ctx->d_rec[cur]);
  smpc::launch_mono_prep<R>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, static_cast<R*>(ctx->d_mpos),
                            static_cast<R*>(ctx->d_mvel), ctx->d_mkey, ctx->d_mimg, ctx->d_count,
                            ctx->d_err, ctx->opt.mono_bin, strict, ctx->d_frames, ctx->rot_c,
                            ctx->rot_s, ctx->mono_chunks, ctx->st);
  smpc::launch_fluid_bin<R>(ctx->d_bin_tiles, ctx->n_bin_tiles, ctx->d_reps, ctx->d_dyn,
                            ctx->d_frames, rec_in, ctx->d_keys, ctx->d_count, ctx->d_err, strict,
                            ctx->opt.angular_momentum ? -1 : ctx->var_bin,
                            ctx->packed_keys ? 1 : 0, static_cast<R*>(ctx->d_frame), ctx->st);
  ctx->frame_ok = ctx->d_frame != nullptr;
  smpc::launch_scan(ctx->d_count, ctx->d_off, ctx->d_tsum, ctx->d_grand,
                    static_cast<int>(ctx->total_cells), ctx->st);
  launch_permutation(ctx);
  return SMPC_OK;
}

template <typename R>
int launch_collision(smpc_ctx* ctx, int rng, int cur) {
  launch_binning<R>(ctx, cur);
  smpc::launch_collide<R>(collide_args<R>(ctx, rng, cur), ctx->st);
  return SMPC_OK;
}

template <typename R>
smpc::CollideArgs<R> collide_args(smpc_ctx* ctx, int rng, int cur) {
  const int strict = ctx->opt.strict_cells;
  smpc::CollideArgs<R> a;
  a.variant = ctx->var_col;
  a.frames = ctx->d_frames;
  a.tiles = ctx->d_col_tiles;
  a.n_tiles = ctx->n_col_tiles;
  if (fast_path(ctx)) {
    const int k = tile_set(smpc::collide_variant_cells(ctx->var_col));
    a.tiles = ctx->d_col_tiles_v[k];
    a.n_tiles = ctx->n_col_tiles_v[k];
  }
  a.reps = ctx->d_reps;
  a.dyn = ctx->d_dyn;
  a.off = ctx->d_off;
  a.perm = ctx->d_perm;
  a.st_in = static_cast<const R*>(ctx->d_rec[cur]);
  a.st_out = static_cast<R*>(ctx->d_rec[cur ^ 1]);
  a.mpos = static_cast<R*>(ctx->d_mpos);
  a.mvel = static_cast<R*>(ctx->d_mvel);
  a.mkey = ctx->d_mkey;
  a.mimg = ctx->d_mimg;
  a.inj_gamma = ctx->d_inj;
  a.inj_uphi = ctx->d_inj + ctx->total_cells;
  a.inj_utheta = ctx->d_inj + 2 * ctx->total_cells;
  a.rng = rng;
  a.rot_c = ctx->rot_c;
  a.rot_s = ctx->rot_s;
  a.strict = strict;
  a.mono_bin = ctx->opt.mono_bin;
  a.amc = ctx->opt.angular_momentum ? 1 : 0;
  a.err = ctx->d_err;
  a.frame = ctx->frame_ok ? static_cast<const R*>(ctx->d_frame) : nullptr;
  return a;
}

template <typename R>
int launch_md_steps(smpc_ctx* ctx, int n, int calc_epot, int force_rebuild) {
  if (ctx->total_mono == 0) return SMPC_OK;
  const double adv = ctx->opt.delrx_mode == SMPC_DELRX_PHYSICAL ? 1.0 / ctx->opt.step_update : 1.0;
  for (const smpc::PmdArgs& p : ctx->pmd)
    smpc::launch_pmd_call<R>(p, ctx->d_reps, ctx->d_dyn, static_cast<R*>(ctx->d_mpos),
                             static_cast<R*>(ctx->d_mnext), static_cast<R*>(ctx->d_mvel),
                             static_cast<R*>(ctx->d_mfrc), static_cast<R*>(ctx->d_mver), n, adv,
                             calc_epot, ctx->var_pmd, ctx->st);
  if (!ctx->any_local_md) return SMPC_OK;
  smpc::MdArgs a;
  a.reps = ctx->d_reps;
  a.dyn = ctx->d_dyn;
  a.bond_start = ctx->d_bond_start;
  a.bonds = ctx->d_bonds;
  a.nlist = ctx->d_nlist;
  a.ncount = ctx->d_ncount;
  a.n_mono_total = static_cast<int>(ctx->total_mono);
  a.max_nb = ctx->max_nb;
  a.n_steps = n;
  a.calc_epot = calc_epot;
  a.force_rebuild = force_rebuild;
  a.core_relative = ctx->opt.strict_cells ? 0 : 1;
  a.err = ctx->d_err;
  a.order = ctx->d_md_order;
  a.andersen = ctx->opt.md_thermostat == SMPC_MDTHERMO_ANDERSEN ? 1 : 0;
  a.andersen_nu = ctx->opt.andersen_nu;
  a.and_start = ctx->and_start_dev;
  a.and_mono = ctx->and_mono_dev;
  a.and_vel = ctx->and_vel_dev;
  a.lowe = ctx->opt.md_thermostat == SMPC_MDTHERMO_LOWE_ANDERSEN ? 1 : 0;
  a.lowe_radius = ctx->opt.lowe_radius;
  a.lowe_buf = ctx->d_lowe;
  smpc::launch_md<R>(a, ctx->n_rep, static_cast<R*>(ctx->d_mpos), static_cast<R*>(ctx->d_mvel),
                     static_cast<R*>(ctx->d_mfrc), static_cast<R*>(ctx->d_mver), ctx->var_md,
                     ctx->st, ctx->md_split);
  return SMPC_OK;
}

// Phases of one fused cycle, in launch order (smpc_cycles_profiled).
enum { PH_MD = 0, PH_BEGIN, PH_MONO, PH_BIN, PH_SCAN, PH_PERM, PH_COLLIDE, PH_END, PH_COUNT };

template <typename R>
int profiled_cycle(smpc_ctx* ctx, int cur, cudaEvent_t* ev) {
  const int nsub = ctx->opt.step_update;
  const int strict = ctx->opt.strict_cells;
  const double adv = ctx->opt.delrx_mode == SMPC_DELRX_PHYSICAL ? 1.0 / nsub : 1.0;
  const R* rec_in = static_cast<const R*>(ctx->d_rec[cur]);
  cudaEventRecord(ev[0], ctx->st);
  launch_md_steps<R>(ctx, nsub, 0, 0);
  cudaEventRecord(ev[1 + PH_MD], ctx->st);
  smpc::launch_cycle_begin<R>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, nsub, adv, 1, ctx->st);
  cudaEventRecord(ev[1 + PH_BEGIN], ctx->st);
  smpc::launch_mono_prep<R>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, static_cast<R*>(ctx->d_mpos),
                            static_cast<R*>(ctx->d_mvel), ctx->d_mkey, ctx->d_mimg, ctx->d_count,
                            ctx->d_err, ctx->opt.mono_bin, strict, ctx->d_frames, ctx->rot_c,
                            ctx->rot_s, ctx->mono_chunks, ctx->st);
  cudaEventRecord(ev[1 + PH_MONO], ctx->st);
  smpc::launch_fluid_bin<R>(ctx->d_bin_tiles, ctx->n_bin_tiles, ctx->d_reps, ctx->d_dyn,
                            ctx->d_frames, rec_in, ctx->d_keys, ctx->d_count, ctx->d_err, strict,
                            ctx->opt.angular_momentum ? -1 : ctx->var_bin,
                            ctx->packed_keys ? 1 : 0, static_cast<R*>(ctx->d_frame), ctx->st);
  ctx->frame_ok = ctx->d_frame != nullptr;
  cudaEventRecord(ev[1 + PH_BIN], ctx->st);
  smpc::launch_scan(ctx->d_count, ctx->d_off, ctx->d_tsum, ctx->d_grand,
                    static_cast<int>(ctx->total_cells), ctx->st);
  cudaEventRecord(ev[1 + PH_SCAN], ctx->st);
  launch_permutation(ctx);
  cudaEventRecord(ev[1 + PH_PERM], ctx->st);
  smpc::CollideArgs<R> a = collide_args<R>(ctx, smpc::RNG_PHILOX, cur);
  smpc::launch_collide<R>(a, ctx->st);
  cudaEventRecord(ev[1 + PH_COLLIDE], ctx->st);
  smpc::launch_cycle_end<R>(ctx->d_dyn, ctx->n_rep, ctx->st);
  cudaEventRecord(ev[1 + PH_END], ctx->st);
  return SMPC_OK;
}

template <typename R>
int record_cycle(smpc_ctx* ctx, int cur) {
  const int nsub = ctx->opt.step_update;
  launch_md_steps<R>(ctx, nsub, 0, 0);
  double adv = 1.0;
  if (ctx->opt.delrx_mode == SMPC_DELRX_PHYSICAL) adv = 1.0 / nsub;
  // h is per replica; k_cycle_begin advances delrx by shear*Ly*h*adv per MD step
  smpc::launch_cycle_begin<R>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, nsub, adv, 1, ctx->st);
  launch_collision<R>(ctx, smpc::RNG_PHILOX, cur);
  smpc::launch_cycle_end<R>(ctx->d_dyn, ctx->n_rep, ctx->st);
  return SMPC_OK;
}

template <typename R>
void to_r4(const double* p3, double w, R* out, size_t i) {
  out[4 * i + 0] = static_cast<R>(p3[3 * i + 0]);
  out[4 * i + 1] = static_cast<R>(p3[3 * i + 1]);
  out[4 * i + 2] = static_cast<R>(p3[3 * i + 2]);
  out[4 * i + 3] = static_cast<R>(w);
}

template <typename R>
uint32_t id_of(R w);
template <>
uint32_t id_of<float>(float w) {
  uint32_t u;
  std::memcpy(&u, &w, 4);
  return u;
}
template <>
uint32_t id_of<double>(double w) {  // the low half of the bit pattern (slot_id)
  uint64_t u;
  std::memcpy(&u, &w, 8);
  return u >> 32 ? smpc::SLOT_EMPTY - 1u : static_cast<uint32_t>(u);
}
template <typename R>
R id_to_w(uint32_t id);
template <>
float id_to_w<float>(uint32_t id) {
  float f;
  std::memcpy(&f, &id, 4);
  return f;
}
template <>
double id_to_w<double>(uint32_t id) {
  const uint64_t u = id;
  double w;
  std::memcpy(&w, &u, 8);
  return w;
}

template <typename R>
int set_fluid_t(smpc_ctx* ctx, int rep, const double* pos, const double* vel) {
  const RepInfo& ri = ctx->reps[rep];
  std::vector<R> rec(8 * static_cast<size_t>(ri.slot_cap));
  for (int i = 0; i < ri.slot_cap; ++i) {
    R* p = rec.data() + 8 * static_cast<size_t>(i);
    if (i < ri.n_fluid) {
      for (int d = 0; d < 3; ++d) {
        p[d] = static_cast<R>(pos[3 * static_cast<size_t>(i) + d]);
        p[4 + d] = static_cast<R>(vel[3 * static_cast<size_t>(i) + d]);
      }
      p[3] = id_to_w<R>(static_cast<uint32_t>(i));
      p[7] = R(0);
    } else {
      for (int d = 0; d < 8; ++d) p[d] = R(0);
      p[3] = id_to_w<R>(smpc::SLOT_EMPTY);
    }
  }
  ctx->frame_ok = false;
  CU(cudaMemcpyAsync(static_cast<R*>(ctx->d_rec[ctx->cur]) + 8 * static_cast<size_t>(ri.slot_base),
                     rec.data(), rec.size() * sizeof(R), cudaMemcpyHostToDevice, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

template <typename R>
int get_fluid_t(smpc_ctx* ctx, int rep, double* pos, double* vel) {
  const RepInfo& ri = ctx->reps[rep];
  std::vector<R> rec(8 * static_cast<size_t>(ri.slot_cap));
  CU(cudaMemcpyAsync(rec.data(), static_cast<R*>(ctx->d_rec[ctx->cur]) + 8 * static_cast<size_t>(ri.slot_base),
                     rec.size() * sizeof(R), cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  int seen = 0;
  for (int i = 0; i < ri.slot_cap; ++i) {
    const R* p = rec.data() + 8 * static_cast<size_t>(i);
    const uint32_t id = id_of<R>(p[3]);
    if (id == smpc::SLOT_EMPTY) continue;
    if (id >= static_cast<uint32_t>(ri.n_fluid))
      return fail(ctx, SMPC_E_STATE, "corrupt solvent slot id");
    for (int d = 0; d < 3; ++d) {
      if (pos) pos[3 * static_cast<size_t>(id) + d] = static_cast<double>(p[d]);
      if (vel) vel[3 * static_cast<size_t>(id) + d] = static_cast<double>(p[4 + d]);
    }
    ++seen;
  }
  if (seen != ri.n_fluid)
    return fail(ctx, SMPC_E_DEVICE, "solvent particles lost (" + std::to_string(seen) + " of " +
                                        std::to_string(ri.n_fluid) + "); see smpc_error_word");
  return SMPC_OK;
}

template <typename R>
int set_monomers_t(smpc_ctx* ctx, int rep, const double* pos, const double* vel,
                   const double* force, const double* mass, const int* amphi, const int* anchor) {
  const RepInfo& ri = ctx->reps[rep];
  const size_t n = static_cast<size_t>(ri.n_mono);
  std::vector<R> p(4 * n), v(4 * n), f(4 * n), pv(4 * n);
  ctx->anchor[rep].assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    const int fl = (amphi ? (amphi[i] != 0) : 0) + 2 * (anchor ? (anchor[i] != 0) : 0);
    ctx->anchor[rep][i] = anchor ? (anchor[i] != 0) : 0;
    ctx->h_mass[ri.mono_base + i] = mass ? mass[i] : 1.0;
    ctx->h_flags[ri.mono_base + i] = static_cast<double>(fl);
    to_r4<R>(pos, mass ? mass[i] : 1.0, p.data(), i);
    to_r4<R>(vel, static_cast<double>(fl), v.data(), i);
    if (force) {
      to_r4<R>(force, 0.0, f.data(), i);
    } else {
      for (int d = 0; d < 4; ++d) f[4 * i + d] = R(0);
    }
    to_r4<R>(pos, 0.0, pv.data(), i);
  }
  const size_t off = 4 * static_cast<size_t>(ri.mono_base);
  const size_t bytes = 4 * n * sizeof(R);
  if (n == 0) return SMPC_OK;
  CU(cudaMemcpyAsync(static_cast<R*>(ctx->d_mpos) + off, p.data(), bytes, cudaMemcpyHostToDevice, ctx->st));
  CU(cudaMemcpyAsync(static_cast<R*>(ctx->d_mvel) + off, v.data(), bytes, cudaMemcpyHostToDevice, ctx->st));
  CU(cudaMemcpyAsync(static_cast<R*>(ctx->d_mfrc) + off, f.data(), bytes, cudaMemcpyHostToDevice, ctx->st));
  CU(cudaMemcpyAsync(static_cast<R*>(ctx->d_mver) + off, pv.data(), bytes, cudaMemcpyHostToDevice, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

template <typename R>
int get_monomers_t(smpc_ctx* ctx, int rep, double* pos, double* vel, double* force) {
  const RepInfo& ri = ctx->reps[rep];
  const size_t n = static_cast<size_t>(ri.n_mono);
  if (n == 0) return SMPC_OK;
  std::vector<R> p(4 * n), v(4 * n), f(4 * n);
  const size_t off = 4 * static_cast<size_t>(ri.mono_base);
  const size_t bytes = 4 * n * sizeof(R);
  CU(cudaMemcpyAsync(p.data(), static_cast<R*>(ctx->d_mpos) + off, bytes, cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaMemcpyAsync(v.data(), static_cast<R*>(ctx->d_mvel) + off, bytes, cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaMemcpyAsync(f.data(), static_cast<R*>(ctx->d_mfrc) + off, bytes, cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      if (pos) pos[3 * i + d] = static_cast<double>(p[4 * i + d]);
      if (vel) vel[3 * i + d] = static_cast<double>(v[4 * i + d]);
      if (force) force[3 * i + d] = static_cast<double>(f[4 * i + d]);
    }
  return SMPC_OK;
}

// Device address of a pinned (page-locked, mapped) host array, or null for
// pageable memory: the unpack kernel then reads the caller's arrays over the
// C2C link instead of staging them through a copy (65 -> 15 us per upload of
// 70 k monomers).
// The mapping is used only when this context's device can reach it: the
// allocation was made with that device current, or it is portable (mapped
// into every device's address space). Otherwise the staged copy is taken.
static void* mapped_host(const void* p, int device) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // clear the query's error state
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
  if (at.device == device) return at.devicePointer;
  unsigned flags = 0;
  if (cudaHostGetFlags(&flags, const_cast<void*>(p)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (flags & cudaHostAllocPortable) ? at.devicePointer : nullptr;
}

// All replicas' monomers in one transfer each way (replicas concatenated),
// through pinned staging buffers allocated at creation. Masses and type flags
// (the .w lanes) come from the host copy kept by smpc_set_monomers.
// Every replica's monomers at once: the host arrays are copied as they are
// (DMA at full speed when they are pinned) and converted on the device.
template <typename R>
int monomers_all_t(smpc_ctx* ctx, const double* pos_in, const double* vel_in, double* pos_out,
                   double* vel_out, double* force_out, bool sync = true) {
  const size_t n = static_cast<size_t>(ctx->total_mono);
  if (n == 0) return SMPC_OK;
  const int ni = static_cast<int>(n);
  if (pos_in) {
    const double* dp = static_cast<const double*>(mapped_host(pos_in, ctx->device));
    const double* dv = static_cast<const double*>(mapped_host(vel_in, ctx->device));
    if (!dp || !dv) {  // pageable arrays: through the staging buffer
      CU(cudaMemcpyAsync(ctx->d_dstage, pos_in, 3 * n * sizeof(double), cudaMemcpyHostToDevice,
                         ctx->st));
      CU(cudaMemcpyAsync(ctx->d_dstage + 3 * n, vel_in, 3 * n * sizeof(double),
                         cudaMemcpyHostToDevice, ctx->st));
      dp = ctx->d_dstage;
      dv = ctx->d_dstage + 3 * n;
    }
    smpc::launch_unpack_monomers<R>(dp, dv, ni, static_cast<R*>(ctx->d_mpos),
                                    static_cast<R*>(ctx->d_mvel), ctx->st);
    CU(cudaGetLastError());
    // Periodic boxes decide list rebuilds from the integrated peculiar
    // displacement, which does not see positions set from outside: request a
    // rebuild at substep 1 (parity 1) of the next call.
    const int one = 1;
    for (const smpc::PmdArgs& a : ctx->pmd)
      CU(cudaMemcpyAsync(a.flag + 1, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
    if (sync) CU(cudaStreamSynchronize(ctx->st));  // the host arrays are borrowed for the call only
    return SMPC_OK;
  }
  // outputs go through the staging buffer and the copy engine even when they
  // are pinned: the pack kernel's 8-byte stores straight into host memory made
  // the download slower (83 against 48 us for 70 k monomers), unlike the reads
  smpc::launch_pack_monomers<R>(static_cast<const R*>(ctx->d_mpos), static_cast<const R*>(ctx->d_mvel),
                                force_out ? static_cast<const R*>(ctx->d_mfrc) : nullptr, ni,
                                ctx->d_dstage, ctx->d_dstage + 3 * n, ctx->d_dstage + 6 * n, ctx->st);
  CU(cudaGetLastError());
  if (pos_out)
    CU(cudaMemcpyAsync(pos_out, ctx->d_dstage, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  if (vel_out)
    CU(cudaMemcpyAsync(vel_out, ctx->d_dstage + 3 * n, 3 * n * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->st));
  if (force_out)
    CU(cudaMemcpyAsync(force_out, ctx->d_dstage + 6 * n, 3 * n * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->st));
  if (sync) CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

template <typename R>
int temperature_all_t(smpc_ctx* ctx, double* out) {
  if (!ctx->collided) return fail(ctx, SMPC_E_STATE, "no collision has run yet (no cell lists)");
  const int nt = static_cast<int>(ctx->h_tmp_tiles.size());
  smpc::launch_temperature<R>(ctx->d_tmp_tiles, nt, ctx->d_reps, ctx->d_off, ctx->d_perm,
                              static_cast<R*>(ctx->d_rec[ctx->cur]), static_cast<R*>(ctx->d_mpos),
                              static_cast<R*>(ctx->d_mvel), ctx->d_mimg, ctx->opt.mono_bin,
                              ctx->d_tpart, ctx->st);
  ctx->stage_t.resize(nt);
  CU(cudaMemcpyAsync(ctx->stage_t.data(), ctx->d_tpart, nt * sizeof(TempPartial),
                     cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  std::vector<double> e(ctx->n_rep, 0.0);
  std::vector<unsigned> filled(ctx->n_rep, 0);
  for (int t = 0; t < nt; ++t) {
    e[ctx->h_tmp_tiles[t].rep] += ctx->stage_t[t].ekin;
    filled[ctx->h_tmp_tiles[t].rep] += ctx->stage_t[t].filled;
  }
  for (int r = 0; r < ctx->n_rep; ++r) {
    const unsigned nf = static_cast<unsigned>(ctx->reps[r].n_fluid);
    out[r] = 2. * e[r] / (3. * static_cast<unsigned>(nf - filled[r]));
  }
  return SMPC_OK;
}

template <typename R>
int temperature_t(smpc_ctx* ctx, int rep, double* out) {
  if (!ctx->collided) return fail(ctx, SMPC_E_STATE, "no collision has run yet (no cell lists)");
  // tiles of this replica only
  int first = -1, count = 0;
  for (size_t t = 0; t < ctx->h_tmp_tiles.size(); ++t)
    if (ctx->h_tmp_tiles[t].rep == rep) {
      if (first < 0) first = static_cast<int>(t);
      ++count;
    }
  smpc::launch_temperature<R>(ctx->d_tmp_tiles + first, count, ctx->d_reps, ctx->d_off,
                              ctx->d_perm, static_cast<R*>(ctx->d_rec[ctx->cur]),
                              static_cast<R*>(ctx->d_mpos), static_cast<R*>(ctx->d_mvel),
                              ctx->d_mimg, ctx->opt.mono_bin, ctx->d_tpart, ctx->st);
  std::vector<TempPartial> part(count);
  CU(cudaMemcpyAsync(part.data(), ctx->d_tpart, count * sizeof(TempPartial),
                     cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  double e = 0.0;
  unsigned filled = 0;
  for (auto& p : part) {
    e += p.ekin;
    filled += p.filled;
  }
  const unsigned nf = static_cast<unsigned>(ctx->reps[rep].n_fluid);
  *out = 2. * e / (3. * static_cast<unsigned>(nf - filled));
  return SMPC_OK;
}

std::vector<Tile> make_tiles(const std::vector<RepInfo>& reps, bool cells, int per_tile) {
  std::vector<Tile> t;
  for (size_t r = 0; r < reps.size(); ++r) {
    const int b = cells ? reps[r].cell_base : reps[r].slot_base;
    const int n = cells ? reps[r].n_cell : reps[r].slot_cap;
    for (int s = 0; s < n; s += per_tile) t.push_back(Tile{static_cast<int>(r), b + s, b + std::min(n, s + per_tile), 0});
  }
  return t;
}

template <typename R>
int create_buffers(smpc_ctx* ctx) {
  const size_t S = static_cast<size_t>(ctx->total_slots), M = static_cast<size_t>(ctx->total_mono),
               C = static_cast<size_t>(ctx->total_cells);
  for (int k = 0; k < 2; ++k) CU(dalloc(reinterpret_cast<R**>(&ctx->d_rec[k]), 8 * S));
  if (std::is_same<R, double>::value) CU(dalloc(reinterpret_cast<R**>(&ctx->d_frame), 8 * S));
  CU(dalloc(&ctx->d_keys, S));
  CU(dalloc(&ctx->d_perm, S + M));
  // a sorted position left unwritten (an error case) holds a valid index
  CU(cudaMemset(ctx->d_perm, 0, (S + M) * sizeof(uint32_t)));
  CU(dalloc(&ctx->d_count, C));
  CU(cudaMemset(ctx->d_count, 0, C * sizeof(uint32_t)));
  CU(dalloc(&ctx->d_off, C + 1));
  CU(dalloc(&ctx->d_tsum, static_cast<size_t>(smpc::scan_tile_count(static_cast<int>(C)))));
  CU(dalloc(&ctx->d_grand, 1));
  CU(dalloc(&ctx->d_init_part, static_cast<size_t>(smpc::INIT_PART_DOUBLES)));
  CU(dalloc(reinterpret_cast<R**>(&ctx->d_mpos), 4 * M));
  CU(dalloc(reinterpret_cast<R**>(&ctx->d_mvel), 4 * M));
  CU(dalloc(reinterpret_cast<R**>(&ctx->d_mfrc), 4 * M));
  CU(dalloc(reinterpret_cast<R**>(&ctx->d_mver), 4 * M));
  CU(dalloc(&ctx->d_mkey, M));
  CU(dalloc(&ctx->d_mimg, M));
  CU(dalloc(&ctx->d_ncount, M));
  if (ctx->opt.md_thermostat == SMPC_MDTHERMO_LOWE_ANDERSEN && M > 0)
    CU(cudaMalloc(&ctx->d_lowe, M * smpc::LOWE_MAX * sizeof(smpc::LoweEntry<R>)));
  CU(cudaMemset(ctx->d_ncount, 0, (M ? M : 1) * sizeof(int)));
  {
    // largest replicas first, so the MD kernel's last wave holds small ones
    std::vector<int> order(ctx->n_rep);
    for (int r = 0; r < ctx->n_rep; ++r) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
      return ctx->reps[p].n_mono > ctx->reps[q].n_mono;
    });
    CU(dalloc(&ctx->d_md_order, order.size()));
    CU(cudaMemcpy(ctx->d_md_order, order.data(), order.size() * sizeof(int),
                  cudaMemcpyHostToDevice));
  }
  CU(dalloc(&ctx->d_nlist, static_cast<size_t>(ctx->max_nb) * M));
  CU(dalloc(&ctx->d_bond_start, M + 1));
  CU(cudaMemset(ctx->d_bond_start, 0, (M + 1) * sizeof(int)));
  CU(dalloc(&ctx->d_inj, 3 * C));
  CU(cudaMemset(ctx->d_inj, 0, 3 * C * sizeof(double)));
  CU(dalloc(&ctx->d_dstage, 9 * M));
  ctx->h_mass.assign(M, 1.0);
  ctx->h_flags.assign(M, 0.0);
  return SMPC_OK;
}

int upload_bonds(smpc_ctx* ctx) {
  // undirected CSR over global monomers; entry (partner, anchor flag of the
  // directed bond's source: the core owns its bonds, Molecule.cpp:146)
  const size_t M = static_cast<size_t>(ctx->total_mono);
  std::vector<std::vector<int2>> adj(M);
  for (int r = 0; r < ctx->n_rep; ++r) {
    const int b = ctx->reps[r].mono_base;
    for (size_t k = 0; k < ctx->bsrc[r].size(); ++k) {
      const int s = ctx->bsrc[r][k], d = ctx->bdst[r][k];
      const int anch = ctx->anchor[r].empty() ? 0 : ctx->anchor[r][s];
      adj[b + s].push_back(make_int2(b + d, anch));
      adj[b + d].push_back(make_int2(b + s, anch));
    }
  }
  std::vector<int> start(M + 1, 0);
  std::vector<int2> flat;
  for (size_t i = 0; i < M; ++i) {
    start[i] = static_cast<int>(flat.size());
    flat.insert(flat.end(), adj[i].begin(), adj[i].end());
  }
  start[M] = static_cast<int>(flat.size());
  if (ctx->d_bonds) cudaFree(ctx->d_bonds);
  ctx->d_bonds = nullptr;
  CU(dalloc(&ctx->d_bonds, flat.size()));
  if (!flat.empty())
    CU(cudaMemcpy(ctx->d_bonds, flat.data(), flat.size() * sizeof(int2), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_bond_start, start.data(), (M + 1) * sizeof(int), cudaMemcpyHostToDevice));
  for (smpc::PmdArgs& p : ctx->pmd) p.bonds = ctx->d_bonds;
  if (ctx->d_pamphi) {  // solvophobic flags (vel.w bit 0) for the periodic force loop
    std::vector<uint8_t> am(M);
    for (size_t i = 0; i < M; ++i) am[i] = static_cast<uint8_t>(static_cast<int>(ctx->h_flags[i]) & 1);
    CU(cudaMemcpy(ctx->d_pamphi, am.data(), M, cudaMemcpyHostToDevice));
  }
  return SMPC_OK;
}

void free_all(smpc_ctx* ctx) {
  for (int k = 0; k < 2; ++k) {
    if (ctx->graph[k]) cudaGraphExecDestroy(ctx->graph[k]);
    cudaFree(ctx->d_rec[k]);
  }
  cudaFree(ctx->d_frame);
  for (void* q : ctx->pmd_mem)
    if (q) cudaFree(q);
  ctx->pmd_mem.clear();
  ctx->pmd.clear();
  if (ctx->d_upos) cudaFree(ctx->d_upos);
  if (ctx->d_uvel) cudaFree(ctx->d_uvel);
  if (ctx->d_mnext) cudaFree(ctx->d_mnext);
  if (ctx->d_ana_part) cudaFree(ctx->d_ana_part);
  if (ctx->d_vacf_ring) cudaFree(ctx->d_vacf_ring);
  if (ctx->d_rows_by_rep) cudaFree(ctx->d_rows_by_rep);
  if (ctx->d_stress) cudaFree(ctx->d_stress);
  if (ctx->d_pamphi) cudaFree(ctx->d_pamphi);
  if (ctx->d_lowe) cudaFree(ctx->d_lowe);
  if (ctx->d_and_i) cudaFree(ctx->d_and_i);
  if (ctx->d_and_v) cudaFree(ctx->d_and_v);
  void* ptrs[] = {ctx->d_reps, ctx->d_dyn, ctx->d_bin_tiles, ctx->d_col_tiles, ctx->d_tmp_tiles,
                  ctx->d_tpart, ctx->d_keys, ctx->d_perm, ctx->d_count, ctx->d_off, ctx->d_tsum,
                  ctx->d_grand, ctx->d_mpos, ctx->d_mvel, ctx->d_mfrc, ctx->d_mver, ctx->d_mkey,
                  ctx->d_mimg, ctx->d_bond_start, ctx->d_bonds, ctx->d_nlist, ctx->d_ncount,
                  ctx->d_md_order, ctx->d_inj, ctx->d_err, ctx->d_frames, ctx->d_rep_mols,
                  ctx->d_mols, ctx->d_obs, ctx->d_prof, ctx->d_c6, ctx->d_dstage, ctx->d_mol_obs,
                  ctx->d_mol_rep, ctx->d_init_part};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int k = 0; k < 3; ++k)
    if (ctx->d_col_tiles_v[k]) cudaFree(ctx->d_col_tiles_v[k]);
  if (ctx->dyn_ev) cudaEventDestroy(ctx->dyn_ev);
  if (ctx->h_dyn_pinned) cudaFreeHost(ctx->h_dyn_pinned);
  if (ctx->md_split.fork) cudaEventDestroy(ctx->md_split.fork);
  if (ctx->md_split.join) cudaEventDestroy(ctx->md_split.join);
  if (ctx->md_split.st2) cudaStreamDestroy(ctx->md_split.st2);
  if (ctx->st) cudaStreamDestroy(ctx->st);
}

template <typename R>
int dispatch_collision(smpc_ctx* ctx, int rng) {
  launch_collision<R>(ctx, rng, ctx->cur);
  if (rng == SMPC_RNG_PHILOX) smpc::launch_cycle_end<R>(ctx->d_dyn, ctx->n_rep, ctx->st);
  ctx->cur ^= 1;
  ctx->collided = true;
  std::fill(ctx->sorted.begin(), ctx->sorted.end(), 1);
  return SMPC_OK;
}

// ------------------------------------------------- allocation-free temperatures
// smpc_temperature_all_noalloc: the same per-tile kernel as
// smpc_temperature_all, with its partial sums and the per-replica results in
// this file-scope device array instead of context buffers and host vectors,
// and the per-replica sums done on the device. It is for callers that must
// not allocate while a run is in flight: a driver that has handed the rest of
// the GPU's memory to its own pool (a cudaMalloc can then fail mid-run), or
// one that polls the temperature from a tight loop where cudaFree would
// synchronise the device. Layout: kNoallocMaxTiles TempPartial, then
// kNoallocMaxReps doubles. Every slot a call reads was written earlier in the
// same call, so nothing has to start at zero. There is one array per device
// (per process), shared by all contexts: calls that overlap in time, from two
// threads or on two streams, race on it.
constexpr int kNoallocMaxTiles = 32768;  // 16.7 M cells at 512 cells per tile
constexpr int kNoallocMaxReps = 4096;
constexpr size_t kNoallocScratchBytes =
    kNoallocMaxTiles * sizeof(TempPartial) + kNoallocMaxReps * sizeof(double);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kNoallocMaxDevices = 64;
void* g_noalloc_ptr[kNoallocMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the first call may load the module; it does not allocate).
cudaError_t noalloc_scratch(int device, void** out) {
  if (device < 0 || device >= kNoallocMaxDevices) return cudaErrorInvalidDevice;
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
  return cudaSuccess;
}

// One thread per replica: its tiles' partial sums in tile order, then
// T = 2 E / (3 (N_solvent - filled cells)) (MPC.cpp:405-409), the same FP64
// operations in the same order as the host sum of smpc_temperature_all. The
// tiles are sorted by replica with each replica's tiles contiguous, so the
// first one is found by binary search and only that range is summed.
__global__ void k_temperature_finish(const Tile* tiles, int n_tiles, const RepInfo* reps,
                                     int n_rep, const TempPartial* part, double* out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rep) return;
  int lo = 0, hi = n_tiles;  // first tile with rep >= r
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (tiles[mid].rep < r) lo = mid + 1;
    else hi = mid;
  }
  double e = 0.0;
  unsigned filled = 0;
  for (int t = lo; t < n_tiles && tiles[t].rep == r; ++t) {
    e += part[t].ekin;
    filled += part[t].filled;
  }
  const unsigned nf = static_cast<unsigned>(reps[r].n_fluid);
  out[r] = 2. * e / (3. * static_cast<unsigned>(nf - filled));
}

template <typename R>
int temperature_all_noalloc_t(smpc_ctx* ctx, double* out) {
  void* base = nullptr;
  CU(noalloc_scratch(ctx->device, &base));
  TempPartial* part = static_cast<TempPartial*>(base);
  double* res = reinterpret_cast<double*>(static_cast<unsigned char*>(base) +
                                          kNoallocMaxTiles * sizeof(TempPartial));
  const int nt = static_cast<int>(ctx->h_tmp_tiles.size());
  smpc::launch_temperature<R>(ctx->d_tmp_tiles, nt, ctx->d_reps, ctx->d_off, ctx->d_perm,
                              static_cast<R*>(ctx->d_rec[ctx->cur]), static_cast<R*>(ctx->d_mpos),
                              static_cast<R*>(ctx->d_mvel), ctx->d_mimg, ctx->opt.mono_bin, part,
                              ctx->st);
  k_temperature_finish<<<(ctx->n_rep + 127) / 128, 128, 0, ctx->st>>>(
      ctx->d_tmp_tiles, nt, ctx->d_reps, ctx->n_rep, part, res);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, res, ctx->n_rep * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

int upload_molecules(smpc_ctx* ctx) {
  std::vector<int2> rep_mols(ctx->n_rep), mols;
  std::vector<int> mol_rep;
  for (int r = 0; r < ctx->n_rep; ++r) {
    const std::vector<int>& ms = ctx->mol_start[r];
    const int base = ctx->reps[r].mono_base;
    rep_mols[r] = make_int2(static_cast<int>(mols.size()), static_cast<int>(ms.size()) - 1);
    for (size_t k = 0; k + 1 < ms.size(); ++k) {
      mols.push_back(make_int2(base + ms[k], base + ms[k + 1]));
      mol_rep.push_back(r);
    }
  }
  for (void* q : {static_cast<void*>(ctx->d_rep_mols), static_cast<void*>(ctx->d_mols),
                  static_cast<void*>(ctx->d_mol_obs), static_cast<void*>(ctx->d_mol_rep)})
    if (q) cudaFree(q);
  ctx->d_rep_mols = nullptr;
  ctx->d_mols = nullptr;
  ctx->d_mol_obs = nullptr;
  ctx->d_mol_rep = nullptr;
  ctx->n_mols = static_cast<int>(mols.size());
  CU(dalloc(&ctx->d_mol_obs, static_cast<size_t>(smpc::OBS_PER_REP) * mols.size()));
  CU(dalloc(&ctx->d_mol_rep, mol_rep.size()));
  if (!mol_rep.empty())
    CU(cudaMemcpy(ctx->d_mol_rep, mol_rep.data(), mol_rep.size() * sizeof(int),
                  cudaMemcpyHostToDevice));
  CU(dalloc(&ctx->d_rep_mols, rep_mols.size()));
  CU(dalloc(&ctx->d_mols, mols.size()));
  CU(cudaMemcpy(ctx->d_rep_mols, rep_mols.data(), rep_mols.size() * sizeof(int2),
                cudaMemcpyHostToDevice));
  if (!mols.empty())
    CU(cudaMemcpy(ctx->d_mols, mols.data(), mols.size() * sizeof(int2), cudaMemcpyHostToDevice));
  return SMPC_OK;
}

// Grid buffers and launch arguments of every periodic box: cells of side
// >= r_verlet (Box.cpp:20-25 sizes its grid the same way), PMD_CELL_CAP beads
// each.
int create_periodic_md(smpc_ctx* ctx) {
  const size_t M = static_cast<size_t>(ctx->total_mono);
  for (int r = 0; r < ctx->n_rep; ++r) {
    const RepInfo& ri = ctx->reps[r];
    if (!(ri.flags & smpc::REP_PERIODIC_MD) || ri.n_mono == 0) continue;
    smpc::PmdArgs a{};
    a.rep = r;
    a.base = ri.mono_base;
    a.n = ri.n_mono;
    a.ncell = 1;
    for (int k = 0; k < 3; ++k) {
      a.nc[k] = static_cast<int>(std::floor(ri.L[k] / ri.r_verlet));
      a.ncell *= a.nc[k];
    }
    a.n_blocks = smpc::pmd_block_count(a.n);
    const size_t cells = static_cast<size_t>(a.ncell);
    void *flag = nullptr, *db = nullptr, *ep = nullptr, *slot = nullptr;
    for (int s = 0; s < 2; ++s) {  // grids of even and odd substeps
      void *cnt = nullptr, *items = nullptr;
      CU(cudaMalloc(&cnt, cells * sizeof(uint32_t)));
      ctx->pmd_mem.push_back(cnt);
      CU(cudaMalloc(&items, cells * smpc::PMD_CELL_CAP * sizeof(int)));
      ctx->pmd_mem.push_back(items);
      CU(cudaMemset(cnt, 0, cells * sizeof(uint32_t)));
      a.cnt[s] = static_cast<uint32_t*>(cnt);
      a.items[s] = static_cast<int*>(items);
    }
    CU(cudaMalloc(&flag, 4 * sizeof(int)));
    ctx->pmd_mem.push_back(flag);
    CU(cudaMalloc(&db, sizeof(double)));
    ctx->pmd_mem.push_back(db);
    // per block of k_pmd_forces, whose lanes per bead depend on the precision
    // and the launch-shape variant
    const int force_blocks = smpc::pmd_force_block_count(a.n, smpc::PMD_MAX_LANES);
    CU(cudaMalloc(&ep, static_cast<size_t>(force_blocks) * sizeof(double)));
    ctx->pmd_mem.push_back(ep);
    CU(cudaMalloc(&slot, 4 * sizeof(double)));
    ctx->pmd_mem.push_back(slot);
    CU(cudaMemset(slot, 0, 4 * sizeof(double)));
    void* rows = nullptr;  // the box's Verlet lists, one row of max_nb per bead
    CU(cudaMalloc(&rows, static_cast<size_t>(a.n) * ctx->max_nb * sizeof(int)));
    ctx->pmd_mem.push_back(rows);
    CU(cudaMemset(flag, 0, 4 * sizeof(int)));
    CU(cudaMemset(db, 0, sizeof(double)));
    a.flag = static_cast<int*>(flag);
    a.delrx_build = static_cast<double*>(db);
    a.epot_part = static_cast<double*>(ep);
    a.dl_slot = static_cast<double*>(slot);
    a.nlist = static_cast<int*>(rows);
    a.ncount = ctx->d_ncount;
    a.n_mono_total = static_cast<int>(M);
    a.max_nb = ctx->max_nb;
    a.bond_start = ctx->d_bond_start;
    a.bonds = ctx->d_bonds;
    a.err = ctx->d_err;
    a.andersen = ctx->opt.md_thermostat == SMPC_MDTHERMO_ANDERSEN ? 1 : 0;
    a.andersen_nu = ctx->opt.andersen_nu;
    ctx->pmd.push_back(a);
  }
  {
    std::vector<int*> rows(ctx->n_rep, nullptr);
    for (const smpc::PmdArgs& p : ctx->pmd) rows[p.rep] = p.nlist;
    CU(dalloc(&ctx->d_rows_by_rep, rows.size()));
    CU(cudaMemcpy(ctx->d_rows_by_rep, rows.data(), rows.size() * sizeof(int*),
                  cudaMemcpyHostToDevice));
    CU(dalloc(&ctx->d_stress, 12 * static_cast<size_t>(ctx->n_rep)));
  }
  if (!ctx->pmd.empty()) {
    CU(cudaMalloc(&ctx->d_pamphi, M));
    CU(cudaMemset(ctx->d_pamphi, 0, M));
    for (smpc::PmdArgs& p : ctx->pmd) p.amphi = ctx->d_pamphi;
    CU(cudaMalloc(&ctx->d_upos, 4 * M * ctx->real_size));
    CU(cudaMalloc(&ctx->d_uvel, 4 * M * ctx->real_size));
    CU(cudaMalloc(&ctx->d_mnext, 4 * M * ctx->real_size));
  }
  return SMPC_OK;
}

}  // namespace

extern "C" {

int smpc_create(const smpc_replica_desc* descs, int n_rep, const smpc_options* opt,
                smpc_ctx** out) {
  if (!descs || n_rep <= 0 || !opt || !out) return SMPC_E_ARG;
  *out = nullptr;
  smpc_ctx* ctx = new smpc_ctx();
  ctx->opt = *opt;
  if (ctx->opt.step_update <= 0) ctx->opt.step_update = 1;
  if (ctx->opt.max_neighbors > 0) ctx->max_nb = ctx->opt.max_neighbors;
  ctx->n_rep = n_rep;
  ctx->sorted.assign(n_rep, 0);
  ctx->device = opt->device;
  ctx->real_size = opt->precision == SMPC_FP64 ? 8 : 4;
  ctx->rot_c = std::cos(130.0 * M_PI / 180.0);  // MPC.cpp:23-24
  ctx->rot_s = std::sin(130.0 * M_PI / 180.0);
  auto bail = [&](int code, const std::string& msg) {
    // creation failed: report through stderr-free path and release everything
    free_all(ctx);
    delete ctx;
    (void)msg;
    return code;
  };
  if (opt->precision != SMPC_FP64 && opt->precision != SMPC_FP32) return bail(SMPC_E_ARG, "precision");
  if (opt->md_thermostat != SMPC_MDTHERMO_NONE && opt->md_thermostat != SMPC_MDTHERMO_ANDERSEN &&
      opt->md_thermostat != SMPC_MDTHERMO_LOWE_ANDERSEN)
    return bail(SMPC_E_ARG, "md thermostat");
  if (opt->md_thermostat != SMPC_MDTHERMO_NONE && !(opt->andersen_nu >= 0))
    return bail(SMPC_E_ARG, "md thermostat frequency");
  const bool lowe = opt->md_thermostat == SMPC_MDTHERMO_LOWE_ANDERSEN;
  if (lowe && !(opt->lowe_radius > 0)) return bail(SMPC_E_ARG, "Lowe-Andersen radius");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return bail(SMPC_E_CUDA, "cudaSetDevice");
  long long cells = 0, slots = 0, mono = 0;
  for (int r = 0; r < n_rep; ++r) {
    const smpc_replica_desc& d = descs[r];
    if (d.L[0] <= 0 || d.L[1] <= 0 || d.L[2] <= 0 || d.n_fluid < 0 || d.n_mono < 0)
      return bail(SMPC_E_ARG, "replica geometry");
    if (d.flags & ~SMPC_REPLICA_PERIODIC_MD) return bail(SMPC_E_ARG, "replica flags");
    const bool periodic = (d.flags & SMPC_REPLICA_PERIODIC_MD) != 0;
    if (!periodic && d.n_mono > smpc::md_max_monomers())
      return bail(SMPC_E_UNSUPPORTED, "too many monomers");
    if (lowe && periodic && d.n_mono > 0)
      return bail(SMPC_E_UNSUPPORTED, "Lowe-Andersen on a periodic box");
    // pairs inside the radius must be in the Verlet lists, which hold every
    // pair inside r_cut at any substep
    if (lowe && d.n_mono > 0 && opt->lowe_radius > d.r_cut)
      return bail(SMPC_E_ARG, "Lowe-Andersen radius above r_cut");
    if (periodic) {
      if (opt->mono_bin != SMPC_MONOBIN_WRAPPED)
        return bail(SMPC_E_ARG, "periodic MD needs wrapped monomer binning");
      for (int k = 0; k < 3; ++k)
        if (!(d.r_verlet > 0) || d.L[k] < 3.0 * d.r_verlet)
          return bail(SMPC_E_UNSUPPORTED, "periodic MD needs every box edge >= 3 r_verlet");
    }
    RepInfo ri{};
    for (int k = 0; k < 3; ++k) ri.L[k] = d.L[k];
    ri.n_cell = d.L[0] * d.L[1] * d.L[2];
    ri.cell_base = static_cast<int>(cells);
    ri.slot_base = static_cast<int>(slots);
    ri.slot_cap = d.n_fluid + d.n_mono;
    ri.n_fluid = d.n_fluid;
    ri.mono_base = static_cast<int>(mono);
    ri.n_mono = d.n_mono;
    ri.mol0_size = periodic ? 0 : d.mol0_size;  // no recentring in a periodic box
    ri.flags = periodic ? smpc::REP_PERIODIC_MD : 0;
    if (!periodic && d.n_mono > 0) ctx->any_local_md = true;
    if (ri.mol0_size == 0)
      ctx->mono_chunks = std::max(ctx->mono_chunks, std::min(1024, (d.n_mono + 1023) / 1024));
    ri.shear = d.shear;
    ri.kT = d.kT;
    ri.h = d.h;
    ri.md_dt = d.md_dt;
    ri.lambda = d.lambda;
    ri.r_cut = d.r_cut;
    ri.r_verlet = d.r_verlet;
    ri.solvent_mass = d.solvent_mass > 0 ? d.solvent_mass : 1.0;
    ri.seed = d.seed;
    ri.potential = d.potential;
    ri.n_sub = ctx->opt.step_update;
    cells += ri.n_cell;
    slots += ri.slot_cap;
    mono += ri.n_mono;
    ctx->reps.push_back(ri);
    RepDyn dn{};
    dn.h = d.h;
    ctx->dyn.push_back(dn);
  }
  if (slots + mono >= 0x7FFFFFFFll || cells >= 0x7FFFFFFFll) return bail(SMPC_E_UNSUPPORTED, "too large");
  ctx->total_cells = cells;
  ctx->total_slots = slots;
  ctx->total_mono = mono;
  ctx->bsrc.resize(n_rep);
  ctx->bdst.resize(n_rep);
  ctx->anchor.resize(n_rep);
  if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->md_split.st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->md_split.fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->md_split.join, cudaEventDisableTiming) != cudaSuccess)
    return bail(SMPC_E_CUDA, "stream");
  if (cudaMallocHost(reinterpret_cast<void**>(&ctx->h_dyn_pinned),
                     sizeof(RepDyn) * static_cast<size_t>(n_rep)) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->dyn_ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(SMPC_E_CUDA, "pinned staging");
  // replicas above 512 monomers lead the MD order (it sorts by size)
  for (int r = 0; r < n_rep; ++r)
    if (ctx->reps[r].n_mono > 512) ++ctx->md_split.n_big;
  {
    // Few replicas: each one's MD on a cluster of SMs (k_md_cluster: always in
    // FP64, whose per-SM rate one CTA cannot get past; an autotuner candidate
    // in FP32). Many replicas: one CTA per replica already fills the GPU.
    int sms = 0, local = 0, biggest = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    for (int r = 0; r < n_rep; ++r)
      if (!(ctx->reps[r].flags & smpc::REP_PERIODIC_MD) && ctx->reps[r].n_mono > 0) {
        ++local;
        biggest = std::max(biggest, ctx->reps[r].n_mono);
      }
    const int cs = opt->precision == SMPC_FP64 ? smpc::md_cluster_size<double>()
                                               : smpc::md_cluster_size<float>();
    if (cs > 0 && local > 0 && local * cs <= sms && biggest <= smpc::MD_CLUSTER_CAP_HOST &&
        opt->md_thermostat != SMPC_MDTHERMO_LOWE_ANDERSEN)
      ctx->md_split.cluster = cs;
  }
  int rc = opt->precision == SMPC_FP64 ? create_buffers<double>(ctx) : create_buffers<float>(ctx);
  if (rc) return bail(rc, ctx->err);
  const int ct = opt->precision == SMPC_FP64 ? smpc::collide_cells_per_tile<double>()
                                             : smpc::collide_cells_per_tile<float>();
  std::vector<Tile> bin =
      make_tiles(ctx->reps, false, smpc::fluid_slots_per_tile(opt->precision == SMPC_FP64));
  std::vector<Tile> col = make_tiles(ctx->reps, true, ct);
  ctx->h_tmp_tiles = make_tiles(ctx->reps, true, smpc::temperature_cells_per_tile());
  ctx->n_bin_tiles = static_cast<int>(bin.size());
  for (const Tile& t : bin) ctx->bin_tile_rep.push_back(t.rep);
  ctx->n_col_tiles = static_cast<int>(col.size());
  bool ok = dalloc(&ctx->d_reps, n_rep) == cudaSuccess && dalloc(&ctx->d_dyn, n_rep) == cudaSuccess &&
            dalloc(&ctx->d_bin_tiles, bin.size()) == cudaSuccess &&
            dalloc(&ctx->d_col_tiles, col.size()) == cudaSuccess &&
            dalloc(&ctx->d_tmp_tiles, ctx->h_tmp_tiles.size()) == cudaSuccess &&
            dalloc(&ctx->d_tpart, ctx->h_tmp_tiles.size()) == cudaSuccess &&
            dalloc(&ctx->d_err, 1) == cudaSuccess && dalloc(&ctx->d_frames, n_rep) == cudaSuccess;
  if (!ok) return bail(SMPC_E_CUDA, "alloc");
  ok = cudaMemcpy(ctx->d_reps, ctx->reps.data(), n_rep * sizeof(RepInfo), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(ctx->d_dyn, ctx->dyn.data(), n_rep * sizeof(RepDyn), cudaMemcpyHostToDevice) == cudaSuccess &&
       (bin.empty() || cudaMemcpy(ctx->d_bin_tiles, bin.data(), bin.size() * sizeof(Tile), cudaMemcpyHostToDevice) == cudaSuccess) &&
       (col.empty() || cudaMemcpy(ctx->d_col_tiles, col.data(), col.size() * sizeof(Tile), cudaMemcpyHostToDevice) == cudaSuccess) &&
       (ctx->h_tmp_tiles.empty() || cudaMemcpy(ctx->d_tmp_tiles, ctx->h_tmp_tiles.data(), ctx->h_tmp_tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice) == cudaSuccess) &&
       cudaMemset(ctx->d_err, 0, sizeof(ErrorState)) == cudaSuccess;
  if (!ok) return bail(SMPC_E_CUDA, "upload");
  ctx->packed_keys = fast_path(ctx);
  for (const RepInfo& ri : ctx->reps)
    if (ri.n_cell > 65536) ctx->packed_keys = false;
  if (fast_path(ctx)) {
    const int cells[3] = {64, 128, 256};
    for (int k = 0; k < 3; ++k) {
      std::vector<Tile> tv = make_tiles(ctx->reps, true, cells[k]);
      ctx->n_col_tiles_v[k] = static_cast<int>(tv.size());
      if (dalloc(&ctx->d_col_tiles_v[k], tv.size()) != cudaSuccess ||
          cudaMemcpy(ctx->d_col_tiles_v[k], tv.data(), tv.size() * sizeof(Tile),
                     cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(SMPC_E_CUDA, "tile tables");
    }
  }
  // molecules: molecule 0 = the first mol0_size monomers (the recentring
  // reference, MPC.cpp:175-176), the rest one more molecule
  ctx->mol_start.resize(n_rep);
  for (int r = 0; r < n_rep; ++r) {
    const int nm = ctx->reps[r].n_mono, m0 = descs[r].mol0_size;
    std::vector<int>& ms = ctx->mol_start[r];
    ms.push_back(0);
    if (nm > 0) {
      if (m0 > 0 && m0 < nm) ms.push_back(m0);
      ms.push_back(nm);
    }
  }
  if (upload_molecules(ctx) != SMPC_OK || dalloc(&ctx->d_obs, static_cast<size_t>(n_rep) * smpc::OBS_PER_REP) != cudaSuccess ||
      dalloc(&ctx->d_c6, 6) != cudaSuccess)
    return bail(SMPC_E_CUDA, "molecule tables");
  if (int rc2 = create_periodic_md(ctx)) return bail(rc2, ctx->err);
  // empty solvent state until smpc_set_fluid: every slot a hole
  for (int r = 0; r < n_rep; ++r) {
    std::vector<double> z(3 * static_cast<size_t>(ctx->reps[r].n_fluid) + 3, 0.0);
    rc = opt->precision == SMPC_FP64 ? set_fluid_t<double>(ctx, r, z.data(), z.data())
                                     : set_fluid_t<float>(ctx, r, z.data(), z.data());
    if (rc) return bail(rc, ctx->err);
  }
  *out = ctx;
  return SMPC_OK;
}

void smpc_destroy(smpc_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  free_all(ctx);
  delete ctx;
}

const char* smpc_last_error(const smpc_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int smpc_n_cells(const smpc_ctx* ctx, int rep) {
  if (!ctx || rep < 0 || rep >= ctx->n_rep) return -1;
  return ctx->reps[rep].n_cell;
}

int smpc_set_fluid(smpc_ctx* ctx, int rep, const double* pos, const double* vel) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (!pos || !vel) return fail(ctx, SMPC_E_ARG, "null buffer");
  ctx->sorted[rep] = 0;
  return ctx->opt.precision == SMPC_FP64 ? set_fluid_t<double>(ctx, rep, pos, vel)
                                         : set_fluid_t<float>(ctx, rep, pos, vel);
}

int smpc_get_fluid(smpc_ctx* ctx, int rep, double* pos, double* vel) {
  if (int rc = check_rep(ctx, rep)) return rc;
  return ctx->opt.precision == SMPC_FP64 ? get_fluid_t<double>(ctx, rep, pos, vel)
                                         : get_fluid_t<float>(ctx, rep, pos, vel);
}

int smpc_set_monomers(smpc_ctx* ctx, int rep, const double* pos, const double* vel,
                      const double* force, const double* mass, const int* amphi,
                      const int* anchor) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (ctx->reps[rep].n_mono > 0 && (!pos || !vel)) return fail(ctx, SMPC_E_ARG, "null buffer");
  ctx->md_ready = false;
  return ctx->opt.precision == SMPC_FP64
             ? set_monomers_t<double>(ctx, rep, pos, vel, force, mass, amphi, anchor)
             : set_monomers_t<float>(ctx, rep, pos, vel, force, mass, amphi, anchor);
}

int smpc_get_monomers(smpc_ctx* ctx, int rep, double* pos, double* vel, double* force) {
  if (int rc = check_rep(ctx, rep)) return rc;
  return ctx->opt.precision == SMPC_FP64 ? get_monomers_t<double>(ctx, rep, pos, vel, force)
                                         : get_monomers_t<float>(ctx, rep, pos, vel, force);
}

int smpc_set_bonds(smpc_ctx* ctx, int rep, int n_bond, const int* src, const int* dst) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (n_bond < 0 || (n_bond > 0 && (!src || !dst))) return fail(ctx, SMPC_E_ARG, "bonds");
  const int n = ctx->reps[rep].n_mono;
  ctx->bsrc[rep].assign(src, src + n_bond);
  ctx->bdst[rep].assign(dst, dst + n_bond);
  for (int k = 0; k < n_bond; ++k)
    if (src[k] < 0 || src[k] >= n || dst[k] < 0 || dst[k] >= n)
      return fail(ctx, SMPC_E_ARG, "bond index out of range");
  ctx->md_ready = false;
  return SMPC_OK;
}

int smpc_init_md(smpc_ctx* ctx) {
  if (!ctx) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  // captured cycles hold the bond table's address, which is about to change
  CU(cudaStreamSynchronize(ctx->st));
  for (int k = 0; k < 2; ++k)
    if (ctx->graph[k]) {
      cudaGraphExecDestroy(ctx->graph[k]);
      ctx->graph[k] = nullptr;
    }
  if (int rc = upload_bonds(ctx)) return rc;
  int rc = ctx->opt.precision == SMPC_FP64 ? launch_md_steps<double>(ctx, 0, 0, 1)
                                           : launch_md_steps<float>(ctx, 0, 0, 1);
  if (rc) return rc;
  CU(cudaGetLastError());
  ctx->md_ready = true;
  return SMPC_OK;
}

int smpc_stage_andersen(smpc_ctx* ctx, int rep, int n_steps, const int* step_start,
                        const int* mono, const double* vel) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (ctx->opt.md_thermostat != SMPC_MDTHERMO_ANDERSEN)
    return fail(ctx, SMPC_E_STATE, "Andersen resets staged without the Andersen thermostat");
  if (ctx->reps[rep].flags & smpc::REP_PERIODIC_MD)
    return fail(ctx, SMPC_E_UNSUPPORTED, "staged Andersen resets on a periodic replica");
  if (n_steps < 1 || !step_start) return fail(ctx, SMPC_E_ARG, "n_steps < 1 or null step_start");
  const int n_mono = ctx->reps[rep].n_mono;
  if (step_start[0] != 0) return fail(ctx, SMPC_E_ARG, "step_start[0] != 0");
  for (int s = 0; s < n_steps; ++s)
    if (step_start[s + 1] < step_start[s])
      return fail(ctx, SMPC_E_ARG, "step_start not non-decreasing");
  const int total = step_start[n_steps];
  if (total > 0 && (!mono || !vel)) return fail(ctx, SMPC_E_ARG, "null reset buffer");
  for (int e = 0; e < total; ++e)
    if (mono[e] < 0 || mono[e] >= n_mono) return fail(ctx, SMPC_E_ARG, "reset monomer out of range");
  if (ctx->and_steps.empty()) {
    ctx->and_steps.assign(ctx->n_rep, -1);
    ctx->and_start_h.resize(ctx->n_rep);
    ctx->and_mono_h.resize(ctx->n_rep);
    ctx->and_vel_h.resize(ctx->n_rep);
  }
  ctx->and_steps[rep] = n_steps;
  ctx->and_start_h[rep].assign(step_start, step_start + n_steps + 1);
  ctx->and_mono_h[rep].assign(mono, mono + total);
  ctx->and_vel_h[rep].assign(vel, vel + 3 * static_cast<size_t>(total));
  return SMPC_OK;
}

// Device table of the staged resets for an n-substep call (layout in
// md_kernels.cuh, MdArgs::and_start); the staged entries are consumed.
static int upload_staged_andersen(smpc_ctx* ctx, int n) {
  std::vector<int> starts(static_cast<size_t>(ctx->n_rep) * (n + 1), -1), monos;
  std::vector<double> vels;
  for (int r = 0; r < ctx->n_rep; ++r) {
    if (ctx->and_steps[r] < 0) continue;
    if (ctx->and_steps[r] != n)
      return fail(ctx, SMPC_E_ARG, "staged Andersen resets cover a different substep count");
    const int base = static_cast<int>(monos.size());
    for (int s = 0; s <= n; ++s)
      starts[static_cast<size_t>(r) * (n + 1) + s] = base + ctx->and_start_h[r][s];
    monos.insert(monos.end(), ctx->and_mono_h[r].begin(), ctx->and_mono_h[r].end());
    vels.insert(vels.end(), ctx->and_vel_h[r].begin(), ctx->and_vel_h[r].end());
    ctx->and_steps[r] = -1;
  }
  const size_t ni = starts.size() + monos.size(), nv = vels.size() > 0 ? vels.size() : 1;
  if (ni > ctx->and_i_cap) {
    if (ctx->d_and_i) CU(cudaFree(ctx->d_and_i));
    ctx->d_and_i = nullptr;
    CU(cudaMalloc(&ctx->d_and_i, ni * sizeof(int)));
    ctx->and_i_cap = ni;
  }
  if (nv > ctx->and_v_cap) {
    if (ctx->d_and_v) CU(cudaFree(ctx->d_and_v));
    ctx->d_and_v = nullptr;
    CU(cudaMalloc(&ctx->d_and_v, nv * sizeof(double)));
    ctx->and_v_cap = nv;
  }
  CU(cudaMemcpyAsync(ctx->d_and_i, starts.data(), starts.size() * sizeof(int),
                     cudaMemcpyHostToDevice, ctx->st));
  if (!monos.empty())
    CU(cudaMemcpyAsync(ctx->d_and_i + starts.size(), monos.data(), monos.size() * sizeof(int),
                       cudaMemcpyHostToDevice, ctx->st));
  if (!vels.empty())
    CU(cudaMemcpyAsync(ctx->d_and_v, vels.data(), vels.size() * sizeof(double),
                       cudaMemcpyHostToDevice, ctx->st));
  // the host tables are locals: wait for the copies before they go
  CU(cudaStreamSynchronize(ctx->st));
  ctx->and_start_dev = ctx->d_and_i;
  ctx->and_mono_dev = ctx->d_and_i + starts.size();
  ctx->and_vel_dev = ctx->d_and_v;
  return SMPC_OK;
}

int smpc_md_substeps(smpc_ctx* ctx, int n, int calc_epot) {
  if (!ctx || n < 0) return SMPC_E_ARG;
  if (ctx->total_mono > 0 && !ctx->md_ready) return fail(ctx, SMPC_E_STATE, "smpc_init_md not called");
  if (n == 0) return SMPC_OK;
  bool staged = false;
  for (int k : ctx->and_steps) staged = staged || k >= 0;
  if (staged)
    if (int rc = upload_staged_andersen(ctx, n)) return rc;
  int rc = ctx->opt.precision == SMPC_FP64 ? launch_md_steps<double>(ctx, n, calc_epot, 0)
                                           : launch_md_steps<float>(ctx, n, calc_epot, 0);
  ctx->and_start_dev = nullptr;
  ctx->and_mono_dev = nullptr;
  ctx->and_vel_dev = nullptr;
  if (rc) return rc;
  CU(cudaGetLastError());
  return SMPC_OK;
}

int smpc_mpc_step(smpc_ctx* ctx, long t, double dt, const smpc_inject* inj) {
  if (!ctx) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  const int su = ctx->opt.step_update;
  const double scale = ctx->opt.delrx_mode == SMPC_DELRX_PHYSICAL ? 1.0 / su : 1.0;
  // MPC.cpp:117-118 on every call, FP64, on the host
  for (int r = 0; r < ctx->n_rep; ++r) {
    RepDyn& dn = ctx->dyn[r];
    const RepInfo& ri = ctx->reps[r];
    dn.delrx += ri.shear * ri.L[1] * (dt * scale);
    dn.delrx -= ri.L[0] * std::round(dn.delrx / ri.L[0]);
    dn.h = dt;
  }
  if (t % su) return upload_host_dyn(ctx);
  const int rng = ctx->opt.rng;
  if (rng == SMPC_RNG_INJECT) {
    if (!inj || !inj->shift || !inj->gamma || !inj->u_phi || !inj->u_theta)
      return fail(ctx, SMPC_E_ARG, "inject mode needs shift, gamma, u_phi and u_theta");
    for (int r = 0; r < ctx->n_rep; ++r)
      for (int d = 0; d < 3; ++d) ctx->dyn[r].shift[d] = inj->shift[3 * r + d];
    const size_t C = static_cast<size_t>(ctx->total_cells);
    CU(cudaMemcpyAsync(ctx->d_inj, inj->gamma, C * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    CU(cudaMemcpyAsync(ctx->d_inj + C, inj->u_phi, C * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    CU(cudaMemcpyAsync(ctx->d_inj + 2 * C, inj->u_theta, C * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  }
  if (int rc = upload_host_dyn(ctx)) return rc;
  if (rng == SMPC_RNG_PHILOX) {
    // device draws the shift from this collision's counter
    if (ctx->opt.precision == SMPC_FP64)
      smpc::launch_cycle_begin<double>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, 0, 0.0, 1, ctx->st);
    else
      smpc::launch_cycle_begin<float>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, 0, 0.0, 1, ctx->st);
  }
  int rc = ctx->opt.precision == SMPC_FP64 ? dispatch_collision<double>(ctx, rng)
                                           : dispatch_collision<float>(ctx, rng);
  if (rc) return rc;
  CU(cudaGetLastError());
  if (rng == SMPC_RNG_INJECT) CU(cudaStreamSynchronize(ctx->st));  // injected buffers are borrowed
  return SMPC_OK;
}

int smpc_mpc_bin(smpc_ctx* ctx, long t, double dt, const double* shift, int* collide_now) {
  if (!ctx || !collide_now) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  *collide_now = 0;
  const int su = ctx->opt.step_update;
  const double scale = ctx->opt.delrx_mode == SMPC_DELRX_PHYSICAL ? 1.0 / su : 1.0;
  for (int r = 0; r < ctx->n_rep; ++r) {  // MPC.cpp:117-118
    RepDyn& dn = ctx->dyn[r];
    const RepInfo& ri = ctx->reps[r];
    dn.delrx += ri.shear * ri.L[1] * (dt * scale);
    dn.delrx -= ri.L[0] * std::round(dn.delrx / ri.L[0]);
    dn.h = dt;
  }
  if (t % su) return upload_host_dyn(ctx);
  if (shift) {
    for (int r = 0; r < ctx->n_rep; ++r)
      for (int d = 0; d < 3; ++d) ctx->dyn[r].shift[d] = shift[3 * r + d];
  } else if (ctx->opt.rng != SMPC_RNG_PHILOX) {
    return fail(ctx, SMPC_E_ARG, "inject mode needs the grid shift");
  }
  if (int rc = upload_host_dyn(ctx)) return rc;
  if (!shift) {
    if (ctx->opt.precision == SMPC_FP64)
      smpc::launch_cycle_begin<double>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, 0, 0.0, 1, ctx->st);
    else
      smpc::launch_cycle_begin<float>(ctx->d_reps, ctx->d_dyn, ctx->n_rep, 0, 0.0, 1, ctx->st);
  }
  if (ctx->opt.precision == SMPC_FP64)
    launch_binning<double>(ctx, ctx->cur);
  else
    launch_binning<float>(ctx, ctx->cur);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(ctx->st));
  ctx->binned = true;
  ctx->bin_philox = shift == nullptr;
  std::fill(ctx->sorted.begin(), ctx->sorted.end(), 0);
  *collide_now = 1;
  return SMPC_OK;
}

int smpc_mpc_collide(smpc_ctx* ctx, const smpc_inject* inj) {
  if (!ctx) return SMPC_E_ARG;
  if (!ctx->binned) return fail(ctx, SMPC_E_STATE, "smpc_mpc_bin has not binned this collision");
  cudaSetDevice(ctx->device);
  const int rng = inj ? SMPC_RNG_INJECT : SMPC_RNG_PHILOX;
  if (rng == SMPC_RNG_INJECT) {
    if (!inj->gamma || !inj->u_phi || !inj->u_theta)
      return fail(ctx, SMPC_E_ARG, "injected draws need gamma, u_phi and u_theta");
    const size_t C = static_cast<size_t>(ctx->total_cells);
    CU(cudaMemcpyAsync(ctx->d_inj, inj->gamma, C * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    CU(cudaMemcpyAsync(ctx->d_inj + C, inj->u_phi, C * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    CU(cudaMemcpyAsync(ctx->d_inj + 2 * C, inj->u_theta, C * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  }
  if (ctx->opt.precision == SMPC_FP64)
    smpc::launch_collide<double>(collide_args<double>(ctx, rng, ctx->cur), ctx->st);
  else
    smpc::launch_collide<float>(collide_args<float>(ctx, rng, ctx->cur), ctx->st);
  if (ctx->bin_philox) {
    if (ctx->opt.precision == SMPC_FP64)
      smpc::launch_cycle_end<double>(ctx->d_dyn, ctx->n_rep, ctx->st);
    else
      smpc::launch_cycle_end<float>(ctx->d_dyn, ctx->n_rep, ctx->st);
  }
  CU(cudaGetLastError());
  if (rng == SMPC_RNG_INJECT) CU(cudaStreamSynchronize(ctx->st));  // borrowed host buffers
  ctx->cur ^= 1;
  ctx->collided = true;
  ctx->binned = false;
  std::fill(ctx->sorted.begin(), ctx->sorted.end(), 1);
  return SMPC_OK;
}

int smpc_cycles(smpc_ctx* ctx, int n) {
  if (!ctx || n < 0) return SMPC_E_ARG;
  if (ctx->opt.rng != SMPC_RNG_PHILOX) return fail(ctx, SMPC_E_STATE, "fused cycles need Philox draws");
  if (ctx->total_mono > 0 && !ctx->md_ready) return fail(ctx, SMPC_E_STATE, "smpc_init_md not called");
  cudaSetDevice(ctx->device);
  // the host mirror of delrx is authoritative between calls
  if (int rc = upload_host_dyn(ctx)) return rc;
  const double scale = ctx->opt.delrx_mode == SMPC_DELRX_PHYSICAL ? 1.0 / ctx->opt.step_update : 1.0;
  for (int i = 0; i < n; ++i) {
    const int cur = ctx->cur;
    if (!ctx->graph[cur]) {
      cudaGraph_t g;
      CU(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
      int rc = ctx->opt.precision == SMPC_FP64 ? record_cycle<double>(ctx, cur)
                                               : record_cycle<float>(ctx, cur);
      cudaError_t e = cudaStreamEndCapture(ctx->st, &g);
      if (rc) return rc;
      if (e != cudaSuccess) return fail(ctx, SMPC_E_CUDA, std::string("capture: ") + cudaGetErrorString(e));
      e = cudaGraphInstantiate(&ctx->graph[cur], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return fail(ctx, SMPC_E_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    }
    CU(cudaGraphLaunch(ctx->graph[cur], ctx->st));
    ctx->cur ^= 1;
    ctx->collided = true;
    std::fill(ctx->sorted.begin(), ctx->sorted.end(), 1);
    // mirror the device's delrx advance (k_cycle_begin), same FP64 operations
    for (int r = 0; r < ctx->n_rep; ++r) {
      const RepInfo& ri = ctx->reps[r];
      RepDyn& dn = ctx->dyn[r];
      for (int s = 0; s < ctx->opt.step_update; ++s) {
        dn.delrx += ri.shear * ri.L[1] * (ri.h * scale);
        dn.delrx -= ri.L[0] * std::round(dn.delrx / ri.L[0]);
      }
      dn.h = ri.h;
    }
  }
  return SMPC_OK;
}

namespace {
int run_profiled(smpc_ctx* ctx, int n, double* phase_ms, double* total_ms) {
  if (int rc = upload_host_dyn(ctx)) return rc;
  const double scale = ctx->opt.delrx_mode == SMPC_DELRX_PHYSICAL ? 1.0 / ctx->opt.step_update : 1.0;
  std::vector<cudaEvent_t> ev(static_cast<size_t>(n) * (PH_COUNT + 1));
  for (auto& e : ev) CU(cudaEventCreate(&e));
  for (int i = 0; i < n; ++i) {
    if (ctx->opt.precision == SMPC_FP64)
      profiled_cycle<double>(ctx, ctx->cur, ev.data() + static_cast<size_t>(i) * (PH_COUNT + 1));
    else
      profiled_cycle<float>(ctx, ctx->cur, ev.data() + static_cast<size_t>(i) * (PH_COUNT + 1));
    ctx->cur ^= 1;
    ctx->collided = true;
    std::fill(ctx->sorted.begin(), ctx->sorted.end(), 1);
    for (int r = 0; r < ctx->n_rep; ++r) {
      const RepInfo& ri = ctx->reps[r];
      RepDyn& dn = ctx->dyn[r];
      for (int s = 0; s < ctx->opt.step_update; ++s) {
        dn.delrx += ri.shear * ri.L[1] * (ri.h * scale);
        dn.delrx -= ri.L[0] * std::round(dn.delrx / ri.L[0]);
      }
      dn.h = ri.h;
    }
  }
  cudaError_t e = cudaStreamSynchronize(ctx->st);
  for (int p = 0; p < PH_COUNT; ++p) phase_ms[p] = 0.0;
  *total_ms = 0.0;
  if (e == cudaSuccess) {
    for (int i = 0; i < n; ++i) {
      cudaEvent_t* c = ev.data() + static_cast<size_t>(i) * (PH_COUNT + 1);
      for (int p = 0; p < PH_COUNT; ++p) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c[p], c[p + 1]);
        phase_ms[p] += ms;
      }
    }
    float tot = 0.f;
    cudaEventElapsedTime(&tot, ev.front(), ev.back());
    *total_ms = tot;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return fail(ctx, SMPC_E_CUDA, cudaGetErrorString(e));
  return SMPC_OK;
}

void drop_graphs(smpc_ctx* ctx) {
  for (int k = 0; k < 2; ++k)
    if (ctx->graph[k]) {
      cudaGraphExecDestroy(ctx->graph[k]);
      ctx->graph[k] = nullptr;
    }
}
}  // namespace

int smpc_cycles_profiled(smpc_ctx* ctx, int n, double* phase_ms, int n_phases, double* total_ms) {
  if (!ctx || n <= 0 || !phase_ms || n_phases < PH_COUNT || !total_ms) return SMPC_E_ARG;
  if (ctx->opt.rng != SMPC_RNG_PHILOX) return fail(ctx, SMPC_E_STATE, "fused cycles need Philox draws");
  if (ctx->total_mono > 0 && !ctx->md_ready) return fail(ctx, SMPC_E_STATE, "smpc_init_md not called");
  cudaSetDevice(ctx->device);
  return run_profiled(ctx, n, phase_ms, total_ms);
}

int smpc_set_variants(smpc_ctx* ctx, int bin, int collide, int md) {
  if (!ctx) return SMPC_E_ARG;
  if (bin < 0 || bin >= smpc::bin_variant_count() || collide < 0 ||
      collide >= smpc::collide_variant_count() || md < 0 || md >= smpc::md_variant_count())
    return fail(ctx, SMPC_E_ARG, "variant index out of range");
  if (bin != ctx->var_bin || collide != ctx->var_col || md != ctx->var_md) drop_graphs(ctx);
  ctx->var_bin = bin;
  ctx->var_col = collide;
  ctx->var_md = md;
  return SMPC_OK;
}

int smpc_set_pmd_variant(smpc_ctx* ctx, int pmd) {
  if (!ctx) return SMPC_E_ARG;
  if (pmd < 0 || pmd >= smpc::pmd_variant_count())
    return fail(ctx, SMPC_E_ARG, "variant index out of range");
  if (pmd != ctx->var_pmd) drop_graphs(ctx);
  ctx->var_pmd = pmd;
  return SMPC_OK;
}

int smpc_get_pmd_variant(const smpc_ctx* ctx, int* pmd) {
  if (!ctx || !pmd) return SMPC_E_ARG;
  *pmd = ctx->var_pmd;
  return SMPC_OK;
}

int smpc_get_variants(const smpc_ctx* ctx, int* bin, int* collide, int* md) {
  if (!ctx) return SMPC_E_ARG;
  if (bin) *bin = ctx->var_bin;
  if (collide) *collide = ctx->var_col;
  if (md) *md = ctx->var_md;
  return SMPC_OK;
}

int smpc_autotune(smpc_ctx* ctx, int cycles, char* report, int report_len) {
  if (!ctx || cycles <= 0) return SMPC_E_ARG;
  if (ctx->opt.rng != SMPC_RNG_PHILOX) return fail(ctx, SMPC_E_STATE, "autotuning runs Philox cycles");
  if (ctx->total_mono > 0 && !ctx->md_ready) return fail(ctx, SMPC_E_STATE, "smpc_init_md not called");
  cudaSetDevice(ctx->device);
  std::string js = "{";
  if (fast_path(ctx)) {
    // the trial cycles run on the live state: keep a full-precision copy of
    // it and put it back afterwards, so tuning leaves the trajectory where it was
    uint64_t snap_bytes = 0;
    if (int rc = smpc_checkpoint_size(ctx, &snap_bytes)) return rc;
    std::vector<unsigned char> snap;
    try {
      snap.resize(snap_bytes);
    } catch (const std::bad_alloc&) {
      return fail(ctx, SMPC_E_ARG, "no host memory for the autotuner's state copy");
    }
    if (int rc = smpc_checkpoint_save(ctx, snap.data(), snap_bytes)) return rc;
    const int var0[4] = {ctx->var_bin, ctx->var_col, ctx->var_md, ctx->var_pmd};
    struct Cat {
      const char* name;
      int phase;
      int count;
      int* var;
      const char* (*label)(int);
    } cats[4] = {{"fluid_bin", PH_BIN, smpc::bin_variant_count(), &ctx->var_bin, smpc::bin_variant_name},
                 {"collide", PH_COLLIDE, smpc::collide_variant_count(), &ctx->var_col,
                  smpc::collide_variant_name},
                 {"md_substeps", PH_MD, smpc::md_variant_count(), &ctx->var_md, smpc::md_variant_name},
                 {"pmd", PH_MD, smpc::pmd_variant_count(), &ctx->var_pmd, smpc::pmd_variant_name}};
    // periodic-MD shapes only where a box runs the periodic MD
    const int n_cats = ctx->pmd.empty() ? 3 : 4;
    double ph[PH_COUNT], tot;
    for (int c = 0; c < n_cats; ++c) {
      int best = 0;
      double best_ms = 1e300;
      js += std::string(c ? ", " : "") + "\"" + cats[c].name + "\": {\"ms_per_cycle\": {";
      for (int v = 0; v < cats[c].count; ++v) {
        *cats[c].var = v;
        drop_graphs(ctx);
        if (int rc = run_profiled(ctx, cycles, ph, &tot)) {
          ctx->var_bin = var0[0];
          ctx->var_col = var0[1];
          ctx->var_md = var0[2];
          ctx->var_pmd = var0[3];
          drop_graphs(ctx);
          smpc_checkpoint_load(ctx, snap.data(), snap_bytes);
          return rc;
        }
        const double ms = ph[cats[c].phase] / cycles;
        char buf[128];
        std::snprintf(buf, sizeof(buf), "%s\"%s\": %.5f", v ? ", " : "", cats[c].label(v), ms);
        js += buf;
        if (ms < best_ms) {
          best_ms = ms;
          best = v;
        }
      }
      *cats[c].var = best;
      drop_graphs(ctx);
      js += std::string("}, \"chosen\": \"") + cats[c].label(best) + "\", \"index\": " +
            std::to_string(best) + "}";
    }
    if (int rc = smpc_checkpoint_load(ctx, snap.data(), snap_bytes)) return rc;
    drop_graphs(ctx);
  }
  js += "}";
  if (report && report_len > 0) {
    std::strncpy(report, js.c_str(), static_cast<size_t>(report_len) - 1);
    report[report_len - 1] = 0;
  }
  return SMPC_OK;
}

int smpc_time_cycles(smpc_ctx* ctx, int n, double* total_ms) {
  if (!ctx || n <= 0 || !total_ms) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  CU(cudaEventRecord(a, ctx->st));
  int rc = smpc_cycles(ctx, n);
  CU(cudaEventRecord(b, ctx->st));
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(ctx, SMPC_E_CUDA, cudaGetErrorString(e));
  *total_ms = ms;
  return SMPC_OK;
}

int smpc_init_solvent(smpc_ctx* ctx, int rep, uint64_t seed, int flags) {
  if (int rc = check_rep(ctx, rep)) return rc;
  cudaSetDevice(ctx->device);
  const RepInfo& ri = ctx->reps[rep];
  ctx->sorted[rep] = 0;
  ctx->frame_ok = false;
  if (ctx->opt.precision == SMPC_FP64)
    smpc::launch_init_solvent<double>(ctx->d_reps, rep, ri.slot_cap,
                                      static_cast<double*>(ctx->d_rec[ctx->cur]), seed, ri.kT,
                                      flags, ctx->d_init_part, ctx->st);
  else
    smpc::launch_init_solvent<float>(ctx->d_reps, rep, ri.slot_cap,
                                     static_cast<float*>(ctx->d_rec[ctx->cur]), seed, ri.kT,
                                     flags, ctx->d_init_part, ctx->st);
  CU(cudaGetLastError());
  return SMPC_OK;
}

int smpc_temperature(smpc_ctx* ctx, int rep, double* out) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (!out) return fail(ctx, SMPC_E_ARG, "null out");
  return ctx->opt.precision == SMPC_FP64 ? temperature_t<double>(ctx, rep, out)
                                         : temperature_t<float>(ctx, rep, out);
}

int smpc_temperature_all(smpc_ctx* ctx, double* out) {
  if (!ctx || !out) return SMPC_E_ARG;
  return ctx->opt.precision == SMPC_FP64 ? temperature_all_t<double>(ctx, out)
                                         : temperature_all_t<float>(ctx, out);
}

int smpc_temperature_all_noalloc(smpc_ctx* ctx, double* out) {
  if (!ctx || !out) return SMPC_E_ARG;
  if (static_cast<long>(ctx->h_tmp_tiles.size()) > kNoallocMaxTiles ||
      ctx->n_rep > kNoallocMaxReps)
    return fail(ctx, SMPC_E_UNSUPPORTED,
                "smpc_temperature_all_noalloc: context has " +
                    std::to_string(ctx->h_tmp_tiles.size()) + " temperature tiles and " +
                    std::to_string(ctx->n_rep) + " replicas; the static scratch holds at most " +
                    std::to_string(kNoallocMaxTiles) + " tiles (512 cells each) and " +
                    std::to_string(kNoallocMaxReps) + " replicas");
  if (!ctx->collided) return fail(ctx, SMPC_E_STATE, "no collision has run yet (no cell lists)");
  cudaSetDevice(ctx->device);
  return ctx->opt.precision == SMPC_FP64 ? temperature_all_noalloc_t<double>(ctx, out)
                                         : temperature_all_noalloc_t<float>(ctx, out);
}

int smpc_set_monomer_state_all(smpc_ctx* ctx, const double* pos, const double* vel) {
  if (!ctx || !pos || !vel) return SMPC_E_ARG;
  return ctx->opt.precision == SMPC_FP64 ? monomers_all_t<double>(ctx, pos, vel, nullptr, nullptr, nullptr)
                                         : monomers_all_t<float>(ctx, pos, vel, nullptr, nullptr, nullptr);
}

int smpc_get_monomer_state_all(smpc_ctx* ctx, double* pos, double* vel, double* force) {
  if (!ctx) return SMPC_E_ARG;
  return ctx->opt.precision == SMPC_FP64 ? monomers_all_t<double>(ctx, nullptr, nullptr, pos, vel, force)
                                         : monomers_all_t<float>(ctx, nullptr, nullptr, pos, vel, force);
}

int smpc_epot(smpc_ctx* ctx, int rep, double* out) {
  if (int rc = check_rep(ctx, rep)) return rc;
  RepDyn dn;
  CU(cudaMemcpyAsync(&dn, ctx->d_dyn + rep, sizeof(RepDyn), cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  *out = dn.epot;
  return SMPC_OK;
}

int smpc_verlet_rebuilds(smpc_ctx* ctx, int rep, int* out) {
  if (int rc = check_rep(ctx, rep)) return rc;
  RepDyn dn;
  CU(cudaMemcpyAsync(&dn, ctx->d_dyn + rep, sizeof(RepDyn), cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  *out = dn.verlet_rebuilds;
  return SMPC_OK;
}

int smpc_delrx(smpc_ctx* ctx, int rep, double* out) {
  if (int rc = check_rep(ctx, rep)) return rc;
  *out = ctx->dyn[rep].delrx;
  return SMPC_OK;
}

int smpc_set_delrx(smpc_ctx* ctx, int rep, double delrx) {
  if (int rc = check_rep(ctx, rep)) return rc;
  ctx->dyn[rep].delrx = delrx;
  return upload_host_dyn(ctx);
}

int smpc_set_collision_counter(smpc_ctx* ctx, uint64_t counter) {
  if (!ctx) return SMPC_E_ARG;
  for (int r = 0; r < ctx->n_rep; ++r) {
    CU(cudaMemcpyAsync(reinterpret_cast<char*>(ctx->d_dyn + r) + offsetof(RepDyn, step), &counter,
                       sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->st));
  }
  CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

int smpc_cell_counts(smpc_ctx* ctx, int rep, unsigned* total, unsigned* fluid) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (!ctx->collided && !ctx->binned) return fail(ctx, SMPC_E_STATE, "no collision has run yet");
  const RepInfo& ri = ctx->reps[rep];
  std::vector<uint32_t> off(ri.n_cell + 1);
  CU(cudaMemcpyAsync(off.data(), ctx->d_off + ri.cell_base, (ri.n_cell + 1) * sizeof(uint32_t),
                     cudaMemcpyDeviceToHost, ctx->st));
  std::vector<uint2> mk(ri.n_mono);
  if (ri.n_mono)
    CU(cudaMemcpyAsync(mk.data(), ctx->d_mkey + ri.mono_base, ri.n_mono * sizeof(uint2),
                       cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  std::vector<unsigned> mono(ri.n_cell, 0);
  for (auto& k : mk)
    if (k.x != smpc::KEY_NONE) mono[k.x - ri.cell_base]++;
  for (int c = 0; c < ri.n_cell; ++c) {
    const unsigned tot = off[c + 1] - off[c];
    if (total) total[c] = tot;
    if (fluid) fluid[c] = tot - mono[c];
  }
  return SMPC_OK;
}

int smpc_cell_members(smpc_ctx* ctx, int rep, int* fluid_cell, int* mono_cell) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (!ctx->sorted[rep])
    return fail(ctx, SMPC_E_STATE, "no collision since the last binning or solvent upload");
  const RepInfo& ri = ctx->reps[rep];
  std::vector<uint32_t> off(ri.n_cell + 1);
  CU(cudaMemcpyAsync(off.data(), ctx->d_off + ri.cell_base, (ri.n_cell + 1) * sizeof(uint32_t),
                     cudaMemcpyDeviceToHost, ctx->st));
  std::vector<uint2> mk(ri.n_mono);
  if (ri.n_mono && mono_cell)
    CU(cudaMemcpyAsync(mk.data(), ctx->d_mkey + ri.mono_base, ri.n_mono * sizeof(uint2),
                       cudaMemcpyDeviceToHost, ctx->st));
  // the id word of every record: after a collision, slot p of the replica holds
  // the particle at sorted position p, so p's cell is the one whose range
  // [off[c], off[c+1]) contains it
  const size_t rec_w = ctx->opt.precision == SMPC_FP64 ? sizeof(double) : sizeof(float);
  std::vector<unsigned char> ids(static_cast<size_t>(ri.slot_cap) * rec_w);
  if (fluid_cell && ri.slot_cap)
    CU(cudaMemcpy2DAsync(ids.data(), rec_w,
                         static_cast<const char*>(ctx->d_rec[ctx->cur]) +
                             (8 * static_cast<size_t>(ri.slot_base) + 3) * rec_w,
                         8 * rec_w, rec_w, ri.slot_cap, cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  if (mono_cell)
    for (int m = 0; m < ri.n_mono; ++m)
      mono_cell[m] = mk[m].x == smpc::KEY_NONE ? -1 : static_cast<int>(mk[m].x - ri.cell_base);
  if (!fluid_cell) return SMPC_OK;
  for (int i = 0; i < ri.n_fluid; ++i) fluid_cell[i] = -1;
  int c = 0;
  for (int i = 0; i < ri.slot_cap; ++i) {
    const uint32_t p = static_cast<uint32_t>(ri.slot_base + i);
    while (c < ri.n_cell && off[c + 1] <= p) ++c;
    uint32_t id;
    if (rec_w == sizeof(double)) {
      double w;
      std::memcpy(&w, ids.data() + i * rec_w, sizeof w);
      id = id_of<double>(w);
    } else {
      float w;
      std::memcpy(&w, ids.data() + i * rec_w, sizeof w);
      id = id_of<float>(w);
    }
    if (id == smpc::SLOT_EMPTY) continue;
    if (id >= static_cast<uint32_t>(ri.n_fluid) || c >= ri.n_cell || fluid_cell[id] != -1)
      return fail(ctx, SMPC_E_STATE, "solvent records are not in cell order");
    fluid_cell[id] = c;
  }
  for (int i = 0; i < ri.n_fluid; ++i)
    if (fluid_cell[i] < 0) return fail(ctx, SMPC_E_DEVICE, "solvent particle missing from the records");
  return SMPC_OK;
}

int smpc_set_molecules(smpc_ctx* ctx, int rep, int n_mol, const int* mol_start) {
  if (int rc = check_rep(ctx, rep)) return rc;
  const int nm = ctx->reps[rep].n_mono;
  if (n_mol < 0 || (n_mol > 0 && !mol_start)) return fail(ctx, SMPC_E_ARG, "molecule table");
  if (n_mol == 0 ? nm != 0 : (mol_start[0] != 0 || mol_start[n_mol] != nm))
    return fail(ctx, SMPC_E_ARG, "molecules must cover the replica's monomers exactly");
  for (int k = 0; k < n_mol; ++k)
    if (mol_start[k + 1] <= mol_start[k]) return fail(ctx, SMPC_E_ARG, "empty or unordered molecule");
  ctx->mol_start[rep].assign(mol_start, mol_start + n_mol + 1);
  if (n_mol == 0) ctx->mol_start[rep].assign(1, 0);
  cudaSetDevice(ctx->device);
  CU(cudaStreamSynchronize(ctx->st));
  return upload_molecules(ctx);
}

}  // extern "C"

namespace {
// Monomer state the observables read: the device arrays, or for contexts with
// periodic boxes their copy with every molecule made whole.
template <typename R>
void observed_monomers(smpc_ctx* ctx, const R** pos, const R** vel) {
  *pos = static_cast<const R*>(ctx->d_mpos);
  *vel = static_cast<const R*>(ctx->d_mvel);
  if (ctx->pmd.empty()) return;
  smpc::launch_unwrap_molecules<R>(ctx->d_reps, ctx->d_dyn, ctx->d_mols, ctx->d_mol_rep,
                                   ctx->n_mols, static_cast<int>(ctx->total_mono),
                                   ctx->d_bond_start, ctx->d_bonds, *pos, *vel,
                                   static_cast<R*>(ctx->d_upos), static_cast<R*>(ctx->d_uvel),
                                   ctx->st);
  *pos = static_cast<const R*>(ctx->d_upos);
  *vel = static_cast<const R*>(ctx->d_uvel);
}

template <typename R>
void mol_observables_t(smpc_ctx* ctx) {
  const R *p, *v;
  observed_monomers<R>(ctx, &p, &v);
  smpc::launch_mol_observables<R>(ctx->d_rep_mols, ctx->d_mols, ctx->n_rep, ctx->n_mols, p, v,
                                  ctx->d_mol_obs, ctx->d_obs, ctx->st);
}

template <typename R>
void velocity_profile_t(smpc_ctx* ctx, int rep, double width, long long kx0, int n_x,
                        long long ky0, int n_y) {
  const R *p, *v;
  observed_monomers<R>(ctx, &p, &v);
  smpc::launch_velocity_profile<R>(ctx->d_reps, ctx->d_rep_mols, ctx->d_mols, rep,
                                   ctx->reps[rep].slot_cap,
                                   static_cast<const R*>(ctx->d_rec[ctx->cur]), p, v,
                                   ctx->dyn[rep].delrx, width, kx0, n_x, ky0, n_y, ctx->d_c6,
                                   ctx->d_prof, ctx->st);
}
}  // namespace

extern "C" {

int smpc_molecule_observables_all(smpc_ctx* ctx, double* out) {
  if (!ctx || !out) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->total_mono > 0 && !ctx->md_ready && !ctx->pmd.empty())
    return fail(ctx, SMPC_E_STATE, "smpc_init_md not called (bonds make periodic molecules whole)");
  if (ctx->opt.precision == SMPC_FP64)
    mol_observables_t<double>(ctx);
  else
    mol_observables_t<float>(ctx);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, ctx->d_obs, static_cast<size_t>(ctx->n_rep) * smpc::OBS_PER_REP * sizeof(double),
                     cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

// The queued part of smpc_cycles_io; returns at the first failure with the
// work queued so far still in flight.
static int cycles_io_queue(smpc_ctx* ctx, int n, const double* pos_in, const double* vel_in,
                           double* pos_out, double* vel_out, double* obs_out) {
  const bool fp64 = ctx->opt.precision == SMPC_FP64;
  if (pos_in) {
    int rc = fp64 ? monomers_all_t<double>(ctx, pos_in, vel_in, nullptr, nullptr, nullptr, false)
                  : monomers_all_t<float>(ctx, pos_in, vel_in, nullptr, nullptr, nullptr, false);
    if (rc) return rc;
  }
  if (int rc = smpc_cycles(ctx, n)) return rc;
  if (pos_out) {
    int rc = fp64 ? monomers_all_t<double>(ctx, nullptr, nullptr, pos_out, vel_out, nullptr, false)
                  : monomers_all_t<float>(ctx, nullptr, nullptr, pos_out, vel_out, nullptr, false);
    if (rc) return rc;
  }
  if (obs_out) {
    if (fp64)
      mol_observables_t<double>(ctx);
    else
      mol_observables_t<float>(ctx);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(obs_out, ctx->d_obs,
                       static_cast<size_t>(ctx->n_rep) * smpc::OBS_PER_REP * sizeof(double),
                       cudaMemcpyDeviceToHost, ctx->st));
  }
  return SMPC_OK;
}

int smpc_cycles_io(smpc_ctx* ctx, int n, const double* pos_in, const double* vel_in,
                   double* pos_out, double* vel_out, double* obs_out) {
  if (!ctx || n < 0) return SMPC_E_ARG;
  if ((pos_in == nullptr) != (vel_in == nullptr) || (pos_out == nullptr) != (vel_out == nullptr))
    return fail(ctx, SMPC_E_ARG, "positions and velocities go together");
  cudaSetDevice(ctx->device);
  const int rc = cycles_io_queue(ctx, n, pos_in, vel_in, pos_out, vel_out, obs_out);
  // Every exit, the failing ones included, waits for what was queued: the
  // pinned input arrays are read in place and the outputs written by queued
  // copies, and the host buffers are borrowed for the call only.
  const cudaError_t e = cudaStreamSynchronize(ctx->st);
  if (rc) return rc;  // the first failure is the one reported
  if (e != cudaSuccess)
    return fail(ctx, SMPC_E_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
  return SMPC_OK;
}

int smpc_velocity_profile(smpc_ctx* ctx, int rep, double width, double* x_out, int n_x,
                          double* y_out, int n_y) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (!(width > 0) || !x_out || !y_out) return fail(ctx, SMPC_E_ARG, "profile width or buffers");
  const RepInfo& ri = ctx->reps[rep];
  const long long kx0 = static_cast<long long>(std::floor(-ri.L[0] / (2.0 * width)));
  const long long ky0 = static_cast<long long>(std::floor(-ri.L[1] / (2.0 * width)));
  const long long need_x = static_cast<long long>(std::floor(ri.L[0] / (2.0 * width))) - kx0 + 1;
  const long long need_y = static_cast<long long>(std::floor(ri.L[1] / (2.0 * width))) - ky0 + 1;
  if (n_x < need_x || n_y < need_y)
    return fail(ctx, SMPC_E_ARG, "profile needs " + std::to_string(need_x) + " x bins and " +
                                     std::to_string(need_y) + " y bins");
  cudaSetDevice(ctx->device);
  const size_t nb = 3 * static_cast<size_t>(n_x + n_y);
  if (nb > ctx->prof_cap) {
    CU(cudaStreamSynchronize(ctx->st));
    if (ctx->d_prof) cudaFree(ctx->d_prof);
    ctx->d_prof = nullptr;
    ctx->prof_cap = 0;
    CU(dalloc(&ctx->d_prof, nb));
    ctx->prof_cap = nb;
  }
  CU(cudaMemsetAsync(ctx->d_prof, 0, nb * sizeof(double), ctx->st));
  if (ctx->total_mono > 0 && !ctx->md_ready && !ctx->pmd.empty())
    return fail(ctx, SMPC_E_STATE, "smpc_init_md not called (bonds make periodic molecules whole)");
  if (ctx->opt.precision == SMPC_FP64)
    velocity_profile_t<double>(ctx, rep, width, kx0, n_x, ky0, n_y);
  else
    velocity_profile_t<float>(ctx, rep, width, kx0, n_x, ky0, n_y);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(x_out, ctx->d_prof, 3 * static_cast<size_t>(n_x) * sizeof(double),
                     cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaMemcpyAsync(y_out, ctx->d_prof + 3 * static_cast<size_t>(n_x),
                     3 * static_cast<size_t>(n_y) * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

int smpc_error_word(smpc_ctx* ctx, unsigned* word, unsigned* info3) {
  if (!ctx) return SMPC_E_ARG;
  ErrorState e;
  CU(cudaMemcpyAsync(&e, ctx->d_err, sizeof(ErrorState), cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaMemsetAsync(ctx->d_err, 0, sizeof(ErrorState), ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  if (word) *word = e.word;
  if (info3)
    for (int k = 0; k < 3; ++k) info3[k] = e.info[k];
  return SMPC_OK;
}

int smpc_synchronize(smpc_ctx* ctx) {
  if (!ctx) return SMPC_E_ARG;
  CU(cudaStreamSynchronize(ctx->st));
  return SMPC_OK;
}

}  // extern "C"

// ------------------------------------------------------------- solvent analyses
namespace {
constexpr int kAnaBlocks = 152 * 4;  // partial sums per analysis pass

int ana_partials(smpc_ctx* ctx, size_t n) {
  if (n <= ctx->ana_part_cap) return SMPC_OK;
  CU(cudaStreamSynchronize(ctx->st));
  if (ctx->d_ana_part) cudaFree(ctx->d_ana_part);
  ctx->d_ana_part = nullptr;
  ctx->ana_part_cap = 0;
  CU(dalloc(&ctx->d_ana_part, n));
  ctx->ana_part_cap = n;
  return SMPC_OK;
}
}  // namespace

extern "C" {

int smpc_fourier_modes(smpc_ctx* ctx, int rep, double box_length, double* out18) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (!out18 || !(box_length > 0)) return fail(ctx, SMPC_E_ARG, "fourier modes: buffer or length");
  cudaSetDevice(ctx->device);
  if (int rc = ana_partials(ctx, 18 * static_cast<size_t>(kAnaBlocks))) return rc;
  const double kwave = 2 * M_PI / box_length;
  if (ctx->opt.precision == SMPC_FP64)
    smpc::launch_fourier_modes<double>(ctx->d_reps, rep, static_cast<const double*>(ctx->d_rec[ctx->cur]),
                                       kwave, ctx->d_ana_part, kAnaBlocks, ctx->st);
  else
    smpc::launch_fourier_modes<float>(ctx->d_reps, rep, static_cast<const float*>(ctx->d_rec[ctx->cur]),
                                      kwave, ctx->d_ana_part, kAnaBlocks, ctx->st);
  CU(cudaGetLastError());
  std::vector<double> part(18 * static_cast<size_t>(kAnaBlocks));
  CU(cudaMemcpyAsync(part.data(), ctx->d_ana_part, part.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  // Fourier_Autocorr: divided by the particle count, component along k removed
  const double n = static_cast<double>(ctx->reps[rep].n_fluid);
  for (int q = 0; q < 18; ++q) {
    double s = 0.0;
    for (int b = 0; b < kAnaBlocks; ++b) s += part[18 * static_cast<size_t>(b) + q];
    out18[q] = n > 0 ? s / n : 0.0;
  }
  for (int j = 0; j < 3; ++j) out18[6 * j + 2 * j] = out18[6 * j + 2 * j + 1] = 0.0;
  return SMPC_OK;
}

int smpc_pressure_tensor_all(smpc_ctx* ctx, double* out) {
  if (!ctx || !out) return SMPC_E_ARG;
  if (ctx->total_mono > 0 && !ctx->md_ready)
    return fail(ctx, SMPC_E_STATE, "smpc_init_md not called (the virial walks the Verlet lists)");
  cudaSetDevice(ctx->device);
  if (int rc = ana_partials(ctx, 6 * static_cast<size_t>(std::max(ctx->n_bin_tiles, 1)))) return rc;
  if (ctx->opt.precision == SMPC_FP64) {
    smpc::launch_kinetic_tensor<double>(ctx->d_bin_tiles, ctx->n_bin_tiles, ctx->d_reps,
                                        static_cast<const double*>(ctx->d_rec[ctx->cur]),
                                        ctx->d_ana_part, ctx->st);
    smpc::launch_mono_stress<double>(ctx->d_reps, ctx->d_dyn, ctx->n_rep,
                                     static_cast<const double*>(ctx->d_mpos),
                                     static_cast<const double*>(ctx->d_mvel), ctx->d_nlist,
                                     ctx->d_ncount, static_cast<int>(ctx->total_mono),
                                     ctx->d_rows_by_rep, ctx->max_nb, ctx->d_bond_start,
                                     ctx->d_bonds, ctx->d_stress, ctx->st);
  } else {
    smpc::launch_kinetic_tensor<float>(ctx->d_bin_tiles, ctx->n_bin_tiles, ctx->d_reps,
                                       static_cast<const float*>(ctx->d_rec[ctx->cur]),
                                       ctx->d_ana_part, ctx->st);
    smpc::launch_mono_stress<float>(ctx->d_reps, ctx->d_dyn, ctx->n_rep,
                                    static_cast<const float*>(ctx->d_mpos),
                                    static_cast<const float*>(ctx->d_mvel), ctx->d_nlist,
                                    ctx->d_ncount, static_cast<int>(ctx->total_mono),
                                    ctx->d_rows_by_rep, ctx->max_nb, ctx->d_bond_start,
                                    ctx->d_bonds, ctx->d_stress, ctx->st);
  }
  CU(cudaGetLastError());
  std::vector<double> part(6 * static_cast<size_t>(ctx->n_bin_tiles));
  std::vector<double> mono(12 * static_cast<size_t>(ctx->n_rep));
  if (!part.empty())
    CU(cudaMemcpyAsync(part.data(), ctx->d_ana_part, part.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaMemcpyAsync(mono.data(), ctx->d_stress, mono.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  // the slot tiles' partial sums, tile by tile into their replicas
  std::vector<double> kin(6 * static_cast<size_t>(ctx->n_rep), 0.0);
  for (int t = 0; t < ctx->n_bin_tiles; ++t)
    for (int k = 0; k < 6; ++k)
      kin[6 * ctx->bin_tile_rep[t] + k] += part[6 * static_cast<size_t>(t) + k];
  for (int q = 0; q < ctx->n_rep; ++q) {
    const RepInfo& ri = ctx->reps[q];
    const double V = static_cast<double>(ri.L[0]) * ri.L[1] * ri.L[2];
    for (int k = 0; k < 6; ++k) {
      out[12 * q + k] = (kin[6 * q + k] + mono[12 * q + k]) / V;
      out[12 * q + 6 + k] = mono[12 * q + 6 + k] / V;
    }
  }
  return SMPC_OK;
}

int smpc_vacf_start(smpc_ctx* ctx, int rep, int n_particles, int entries) {
  if (int rc = check_rep(ctx, rep)) return rc;
  if (n_particles <= 0 || n_particles > ctx->reps[rep].n_fluid || entries <= 0)
    return fail(ctx, SMPC_E_ARG, "vacf: particle count or entries");
  cudaSetDevice(ctx->device);
  CU(cudaStreamSynchronize(ctx->st));
  if (ctx->d_vacf_ring) cudaFree(ctx->d_vacf_ring);
  ctx->d_vacf_ring = nullptr;
  CU(dalloc(&ctx->d_vacf_ring, 3 * static_cast<size_t>(n_particles) * entries));
  if (int rc = ana_partials(ctx, static_cast<size_t>(kAnaBlocks) * entries)) return rc;
  ctx->vacf_rep = rep;
  ctx->vacf_np = n_particles;
  ctx->vacf_entries = entries;
  ctx->vacf_samples = 0;
  ctx->vacf_calcs = 0;
  ctx->vacf_sum.assign(entries, 0.0);
  return SMPC_OK;
}

int smpc_vacf_sample(smpc_ctx* ctx) {
  if (!ctx) return SMPC_E_ARG;
  if (ctx->vacf_rep < 0) return fail(ctx, SMPC_E_STATE, "smpc_vacf_start not called");
  cudaSetDevice(ctx->device);
  const int rep = ctx->vacf_rep, E = ctx->vacf_entries, np = ctx->vacf_np;
  const int slot = static_cast<int>(ctx->vacf_samples % static_cast<uint64_t>(E));
  if (ctx->opt.precision == SMPC_FP64)
    smpc::launch_vacf_sample<double>(ctx->d_reps, rep, ctx->reps[rep].slot_cap,
                                     static_cast<const double*>(ctx->d_rec[ctx->cur]), np, slot,
                                     ctx->d_vacf_ring, ctx->st);
  else
    smpc::launch_vacf_sample<float>(ctx->d_reps, rep, ctx->reps[rep].slot_cap,
                                    static_cast<const float*>(ctx->d_rec[ctx->cur]), np, slot,
                                    ctx->d_vacf_ring, ctx->st);
  ctx->vacf_samples += 1;
  if (ctx->vacf_samples < static_cast<uint64_t>(E)) {
    CU(cudaGetLastError());
    return SMPC_OK;
  }
  // the window is full: Vel_Autocorr_Fluid::calculate() over its samples
  const int first = static_cast<int>((ctx->vacf_samples - E) % static_cast<uint64_t>(E));
  const int nb = std::min(kAnaBlocks, (np + 255) / 256);
  if (ctx->opt.precision == SMPC_FP64)
    smpc::launch_vacf_lags<double>(ctx->d_vacf_ring, np, E, first, ctx->d_ana_part, nb, ctx->st);
  else
    smpc::launch_vacf_lags<float>(ctx->d_vacf_ring, np, E, first, ctx->d_ana_part, nb, ctx->st);
  CU(cudaGetLastError());
  std::vector<double> part(static_cast<size_t>(nb) * E);
  CU(cudaMemcpyAsync(part.data(), ctx->d_ana_part, part.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, ctx->st));
  CU(cudaStreamSynchronize(ctx->st));
  for (int j = 0; j < E; ++j) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[static_cast<size_t>(j) * nb + b];
    ctx->vacf_sum[j] += s;
  }
  ctx->vacf_calcs += 1;
  return SMPC_OK;
}

int smpc_vacf_result(smpc_ctx* ctx, double* lag_sums, uint64_t* calculations) {
  if (!ctx || !lag_sums || !calculations) return SMPC_E_ARG;
  if (ctx->vacf_rep < 0) return fail(ctx, SMPC_E_STATE, "smpc_vacf_start not called");
  for (int j = 0; j < ctx->vacf_entries; ++j) lag_sums[j] = ctx->vacf_sum[j];
  *calculations = ctx->vacf_calcs;
  return SMPC_OK;
}

}  // extern "C"

// ------------------------------------------------------------- checkpoints
// One blob holds everything a context needs to continue a run exactly where it
// was saved: the host mirror and device copy of every replica's dynamic record
// (delrx, grid shift, Philox collision counter, rebuild counter, ...), the
// solvent records in their cell order, the monomer state with its forces,
// Verlet lists and their references, the last collision's cell lists (for
// the observables), bonds, molecules, and the periodic-MD bookkeeping. Every
// section is the context's own bytes (FP32 or FP64), so a restored context
// continues bit for bit. The reference writes lossy text (%f, %7.3f) and draws
// a new random stream on restart (MPC.cpp:57-113, 570-579; Box.cpp:563-602).
namespace {

constexpr char kCkptMagic[8] = {'S', 'M', 'P', 'C', 'C', 'K', 'P', '1'};
// version 2: FP64 solvent records carry the slot id as the low half of the
// .w bit pattern (version 1: as a number)
constexpr uint32_t kCkptVersion = 2;

struct CkptHeader {
  char magic[8];
  uint32_t version;
  uint32_t precision;
  uint32_t n_rep;
  uint32_t step_update;
  uint32_t mono_bin;
  uint32_t delrx_mode;
  uint32_t strict;
  uint32_t max_nb;
  uint32_t cur;
  uint32_t collided;
  uint64_t total_slots;
  uint64_t total_mono;
  uint64_t total_cells;
  uint64_t n_pmd;
};

// Byte stream to a buffer, a file, or nowhere (size count).
struct CkptIo {
  unsigned char* buf = nullptr;      // save into memory
  const unsigned char* in = nullptr; // load from memory
  uint64_t cap = 0;
  uint64_t pos = 0;
  FILE* f = nullptr;
  bool ok = true;
};

void ck_put(CkptIo& io, const void* p, uint64_t n) {
  if (!io.ok || n == 0) {
    io.pos += io.ok ? n : 0;
    return;
  }
  if (io.f) {
    io.ok = std::fwrite(p, 1, n, io.f) == n;
  } else if (io.buf) {
    if (io.pos + n > io.cap) {
      io.ok = false;
      return;
    }
    std::memcpy(io.buf + io.pos, p, n);
  }
  io.pos += n;
}

void ck_get(CkptIo& io, void* p, uint64_t n) {
  if (!io.ok || n == 0) return;
  if (io.f) {
    io.ok = std::fread(p, 1, n, io.f) == n;
  } else {
    if (io.pos + n > io.cap) {
      io.ok = false;
      return;
    }
    std::memcpy(p, io.in + io.pos, n);
  }
  io.pos += n;
}

// device bytes through a bounded host staging buffer
constexpr uint64_t kCkptChunk = 64ull << 20;

int ck_put_dev(smpc_ctx* ctx, CkptIo& io, const void* d, uint64_t n) {
  if (!io.ok || n == 0 || (!io.f && !io.buf)) {
    io.pos += io.ok ? n : 0;
    return SMPC_OK;
  }
  if (io.buf) {  // straight into the caller's buffer
    if (io.pos + n > io.cap) {
      io.ok = false;
      return SMPC_OK;
    }
    CU(cudaMemcpy(io.buf + io.pos, d, n, cudaMemcpyDeviceToHost));
    io.pos += n;
    return SMPC_OK;
  }
  std::vector<unsigned char> stage(std::min(n, kCkptChunk));
  for (uint64_t o = 0; o < n; o += kCkptChunk) {
    const uint64_t k = std::min(kCkptChunk, n - o);
    CU(cudaMemcpy(stage.data(), static_cast<const unsigned char*>(d) + o, k, cudaMemcpyDeviceToHost));
    ck_put(io, stage.data(), k);
  }
  return SMPC_OK;
}

int ck_get_dev(smpc_ctx* ctx, CkptIo& io, void* d, uint64_t n) {
  if (!io.ok || n == 0) return SMPC_OK;
  if (!io.f) {
    if (io.pos + n > io.cap) {
      io.ok = false;
      return SMPC_OK;
    }
    CU(cudaMemcpy(d, io.in + io.pos, n, cudaMemcpyHostToDevice));
    io.pos += n;
    return SMPC_OK;
  }
  std::vector<unsigned char> stage(std::min(n, kCkptChunk));
  for (uint64_t o = 0; o < n && io.ok; o += kCkptChunk) {
    const uint64_t k = std::min(kCkptChunk, n - o);
    ck_get(io, stage.data(), k);
    if (io.ok) CU(cudaMemcpy(static_cast<unsigned char*>(d) + o, stage.data(), k, cudaMemcpyHostToDevice));
  }
  return SMPC_OK;
}

template <typename T>
void ck_put_vec(CkptIo& io, const std::vector<T>& v) {
  const uint64_t n = v.size();
  ck_put(io, &n, sizeof n);
  ck_put(io, v.data(), n * sizeof(T));
}

template <typename T>
void ck_get_vec(CkptIo& io, std::vector<T>& v, uint64_t limit) {
  uint64_t n = 0;
  ck_get(io, &n, sizeof n);
  if (!io.ok || n > limit) {
    io.ok = false;
    return;
  }
  v.resize(n);
  ck_get(io, v.data(), n * sizeof(T));
}

CkptHeader ck_header(const smpc_ctx* ctx) {
  CkptHeader h{};
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = kCkptVersion;
  h.precision = static_cast<uint32_t>(ctx->opt.precision);
  h.n_rep = static_cast<uint32_t>(ctx->n_rep);
  h.step_update = static_cast<uint32_t>(ctx->opt.step_update);
  h.mono_bin = static_cast<uint32_t>(ctx->opt.mono_bin);
  h.delrx_mode = static_cast<uint32_t>(ctx->opt.delrx_mode);
  h.strict = static_cast<uint32_t>(ctx->opt.strict_cells);
  h.max_nb = static_cast<uint32_t>(ctx->max_nb);
  h.cur = static_cast<uint32_t>(ctx->cur);
  h.collided = ctx->collided ? 1u : 0u;
  h.total_slots = static_cast<uint64_t>(ctx->total_slots);
  h.total_mono = static_cast<uint64_t>(ctx->total_mono);
  h.total_cells = static_cast<uint64_t>(ctx->total_cells);
  h.n_pmd = ctx->pmd.size();
  return h;
}

// The device arrays of a checkpoint, in order, with their sizes.
struct CkptArray {
  void* d;
  uint64_t bytes;
};

std::vector<CkptArray> ck_arrays(smpc_ctx* ctx) {
  const uint64_t S = static_cast<uint64_t>(ctx->total_slots), M = static_cast<uint64_t>(ctx->total_mono),
                 C = static_cast<uint64_t>(ctx->total_cells), rs = ctx->real_size;
  std::vector<CkptArray> a = {
      {ctx->d_dyn, ctx->n_rep * sizeof(RepDyn)},
      {ctx->d_rec[ctx->cur], 8 * S * rs},
      {ctx->d_mpos, 4 * M * rs},
      {ctx->d_mvel, 4 * M * rs},
      {ctx->d_mfrc, 4 * M * rs},
      {ctx->d_mver, 4 * M * rs},
      {ctx->d_nlist, static_cast<uint64_t>(ctx->max_nb) * M * sizeof(int)},
      {ctx->d_ncount, M * sizeof(int)},
      {ctx->d_off, (C + 1) * sizeof(uint32_t)},
      {ctx->d_perm, (S + M) * sizeof(uint32_t)},
      {ctx->d_mkey, M * sizeof(uint2)},
      {ctx->d_mimg, M * sizeof(int)},
  };
  for (const smpc::PmdArgs& p : ctx->pmd) {
    a.push_back({p.flag, 4 * sizeof(int)});
    a.push_back({p.delrx_build, sizeof(double)});
    a.push_back({p.dl_slot, 4 * sizeof(double)});
    a.push_back({p.nlist, static_cast<uint64_t>(p.n) * ctx->max_nb * sizeof(int)});
  }
  return a;
}

int ck_save(smpc_ctx* ctx, CkptIo& io) {
  if (ctx->binned) return fail(ctx, SMPC_E_STATE, "a collision is binned but not collided");
  CU(cudaStreamSynchronize(ctx->st));
  const CkptHeader h = ck_header(ctx);
  ck_put(io, &h, sizeof h);
  ck_put(io, ctx->reps.data(), ctx->n_rep * sizeof(RepInfo));
  ck_put(io, ctx->dyn.data(), ctx->n_rep * sizeof(RepDyn));
  ck_put(io, ctx->sorted.data(), ctx->sorted.size());
  for (int r = 0; r < ctx->n_rep; ++r) {
    ck_put_vec(io, ctx->bsrc[r]);
    ck_put_vec(io, ctx->bdst[r]);
    ck_put_vec(io, ctx->anchor[r]);
    ck_put_vec(io, ctx->mol_start[r]);
  }
  ck_put_vec(io, ctx->h_mass);
  ck_put_vec(io, ctx->h_flags);
  const uint8_t md = ctx->md_ready ? 1 : 0;
  ck_put(io, &md, 1);
  for (const CkptArray& a : ck_arrays(ctx))
    if (int rc = ck_put_dev(ctx, io, a.d, a.bytes)) return rc;
  if (!io.ok) return fail(ctx, SMPC_E_ARG, "checkpoint buffer too small or write failed");
  return SMPC_OK;
}

int ck_load(smpc_ctx* ctx, CkptIo& io) {
  if (ctx->binned) return fail(ctx, SMPC_E_STATE, "a collision is binned but not collided");
  CU(cudaStreamSynchronize(ctx->st));
  CkptHeader h{};
  ck_get(io, &h, sizeof h);
  if (!io.ok || std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != kCkptVersion)
    return fail(ctx, SMPC_E_ARG, "not a checkpoint of this format");
  CkptHeader mine = ck_header(ctx);
  mine.cur = h.cur;
  mine.collided = h.collided;
  if (std::memcmp(&h, &mine, sizeof h) != 0 || h.cur > 1)
    return fail(ctx, SMPC_E_ARG, "checkpoint of a context with other replicas or options");
  std::vector<RepInfo> reps(ctx->n_rep);
  ck_get(io, reps.data(), reps.size() * sizeof(RepInfo));
  if (!io.ok || std::memcmp(reps.data(), ctx->reps.data(), reps.size() * sizeof(RepInfo)) != 0)
    return fail(ctx, SMPC_E_ARG, "checkpoint of a context with other replicas");
  std::vector<RepDyn> dyn(ctx->n_rep);
  std::vector<uint8_t> sorted(ctx->n_rep);
  ck_get(io, dyn.data(), dyn.size() * sizeof(RepDyn));
  ck_get(io, sorted.data(), sorted.size());
  std::vector<std::vector<int>> bsrc(ctx->n_rep), bdst(ctx->n_rep), anchor(ctx->n_rep),
      mol(ctx->n_rep);
  const uint64_t M = static_cast<uint64_t>(ctx->total_mono);
  for (int r = 0; r < ctx->n_rep; ++r) {
    const uint64_t n = static_cast<uint64_t>(ctx->reps[r].n_mono);
    ck_get_vec(io, bsrc[r], 4 * n + 16);
    ck_get_vec(io, bdst[r], 4 * n + 16);
    ck_get_vec(io, anchor[r], n);
    ck_get_vec(io, mol[r], n + 1);
    for (size_t k = 0; io.ok && k < bsrc[r].size(); ++k)
      if (k >= bdst[r].size() || bsrc[r][k] < 0 || static_cast<uint64_t>(bsrc[r][k]) >= n ||
          bdst[r][k] < 0 || static_cast<uint64_t>(bdst[r][k]) >= n)
        io.ok = false;
    if (io.ok && (mol[r].empty() || mol[r].front() != 0 ||
                  (n > 0 && static_cast<uint64_t>(mol[r].back()) != n)))
      io.ok = false;
  }
  std::vector<double> mass, flags;
  ck_get_vec(io, mass, M);
  ck_get_vec(io, flags, M);
  uint8_t md = 0;
  ck_get(io, &md, 1);
  if (!io.ok || mass.size() != M || flags.size() != M)
    return fail(ctx, SMPC_E_ARG, "truncated or inconsistent checkpoint");
  // from here the context's state is replaced
  for (int k = 0; k < 2; ++k)
    if (ctx->graph[k]) {
      cudaGraphExecDestroy(ctx->graph[k]);
      ctx->graph[k] = nullptr;
    }
  ctx->cur = static_cast<int>(h.cur);
  for (const CkptArray& a : ck_arrays(ctx))
    if (int rc = ck_get_dev(ctx, io, a.d, a.bytes)) return rc;
  if (!io.ok) return fail(ctx, SMPC_E_ARG, "truncated checkpoint (context state undefined)");
  ctx->collided = h.collided != 0;
  ctx->binned = false;
  ctx->frame_ok = false;
  ctx->dyn = dyn;
  ctx->sorted = sorted;
  ctx->bsrc = bsrc;
  ctx->bdst = bdst;
  ctx->anchor = anchor;
  ctx->mol_start = mol;
  ctx->h_mass = mass;
  ctx->h_flags = flags;
  if (int rc = upload_molecules(ctx)) return rc;
  if (int rc = upload_bonds(ctx)) return rc;
  ctx->md_ready = md != 0;
  return SMPC_OK;
}

}  // namespace

extern "C" {

int smpc_checkpoint_size(smpc_ctx* ctx, uint64_t* bytes) {
  if (!ctx || !bytes) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  CkptIo io;  // counts only
  if (int rc = ck_save(ctx, io)) return rc;
  *bytes = io.pos;
  return SMPC_OK;
}

int smpc_checkpoint_save(smpc_ctx* ctx, void* buf, uint64_t cap) {
  if (!ctx || !buf) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  CkptIo io;
  io.buf = static_cast<unsigned char*>(buf);
  io.cap = cap;
  return ck_save(ctx, io);
}

int smpc_checkpoint_load(smpc_ctx* ctx, const void* buf, uint64_t len) {
  if (!ctx || !buf) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  CkptIo io;
  io.in = static_cast<const unsigned char*>(buf);
  io.cap = len;
  return ck_load(ctx, io);
}

int smpc_checkpoint_write(smpc_ctx* ctx, const char* path) {
  if (!ctx || !path) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(ctx, SMPC_E_ARG, std::string("cannot open ") + path + " for writing");
  CkptIo io;
  io.f = f;
  int rc = ck_save(ctx, io);
  if (std::fclose(f) != 0 && rc == SMPC_OK) rc = fail(ctx, SMPC_E_ARG, "checkpoint write failed");
  return rc;
}

int smpc_checkpoint_read(smpc_ctx* ctx, const char* path) {
  if (!ctx || !path) return SMPC_E_ARG;
  cudaSetDevice(ctx->device);
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(ctx, SMPC_E_ARG, std::string("cannot open ") + path);
  CkptIo io;
  io.f = f;
  const int rc = ck_load(ctx, io);
  std::fclose(f);
  return rc;
}

}  // extern "C"
