// Device-side data layout shared by the host context (smpc_capi.cu) and the
// kernels (mpc_kernels.cuh, md_kernels.cuh).
//
// HBM layout (all replicas of a context concatenated):
//   solvent slots   pos[4*S], vel[4*S] of Real, two copies (ping-pong);
//                   pos.w holds the particle id (uint32 bits for float,
//                   an exact integer for double), SLOT_EMPTY marks a hole.
//                   Replica r owns slots [slot_base, slot_base + n_fluid + n_mono):
//                   after each collision its solvent is written back in cell
//                   order, the n_mono slots taken by monomers stay empty.
//   keys            uint2 per slot and per monomer: (global cell, rank in cell)
//   cells           count[C], off[C+1] (exclusive scan), per-tile scan sums
//   perm            uint32 per sorted position: source slot, or MONO_BIT|monomer
//   monomers        pos/vel/force/verlet-pos as Real4 (pos.w = mass,
//                   vel.w = amphi + 2*anchor), CSR bond lists, Verlet lists
#pragma once
#include <stdint.h>

namespace smpc {

constexpr uint32_t SLOT_EMPTY = 0xFFFFFFFFu;
constexpr uint32_t MONO_BIT = 0x80000000u;
constexpr uint32_t KEY_NONE = 0xFFFFFFFFu;

// error word bits (host maps them to messages; none of them traps)
enum : uint32_t {
  ERR_FLUID_CELL = 1u,     // solvent cell index out of range (MPC.cpp:211-219)
  ERR_MONO_CELL = 2u,      // monomer cell index out of range (MPC.cpp:227-234)
  ERR_NEIGHBOR_OVF = 4u,   // Verlet list capacity exceeded
  ERR_NONFINITE = 8u,      // non-finite velocity after a collision
  ERR_TILE_OVF = 16u,      // collide tile larger than its register cache (handled, slow path)
  ERR_GAMMA_ITERS = 32u,   // gamma sampler hit its iteration limit
  ERR_FENE = 64u,          // FENE bond stretched beyond R0 (Potentials.h:29,50)
  ERR_KEY_MISMATCH = 128u, // collide recomputed a different cell than binning (never expected)
  ERR_FIXPOINT = 256u      // FP32 cell sum term outside the fixed-point range (precision.cuh)
};

enum : int { POT_REF4824 = 0, POT_LJ126 = 1 };
enum : int { MONOBIN_REFERENCE = 0, MONOBIN_WRAPPED = 1 };
enum : int { RNG_INJECT = 0, RNG_PHILOX = 1 };
enum : int { REP_PERIODIC_MD = 1 };  // smpc.h SMPC_REPLICA_PERIODIC_MD

// Static per-replica description (uploaded once).
struct RepInfo {
  int L[3];
  int n_cell;          // L0*L1*L2
  int cell_base;       // first global cell
  int slot_base;       // first solvent slot
  int slot_cap;        // n_fluid + n_mono
  int n_fluid;
  int mono_base;
  int n_mono;
  int mol0_size;       // monomers of molecule 0 (recentring reference)
  int flags;           // REP_* bits
  double shear;
  double kT;
  double h;            // collision step (streaming time)
  double md_dt;
  double lambda;
  double r_cut;
  double r_verlet;
  double solvent_mass;
  unsigned long long seed;
  int potential;
  int n_sub;
};

// Per-collision per-replica dynamic values.
struct RepDyn {
  // host-owned in step mode (written by one strided copy of the leading bytes)
  double delrx;          // Lees-Edwards image offset (FP64 always)
  double shift[3];       // random grid shift of this collision
  double h;              // streaming time of this collision (MPC::step dt)
  // device-owned
  double com[3];         // recentring: star-0 centre of mass (MPC::check_bounds)
  double comv[3];
  int recentre;          // 1 when MPC::check_bounds fired this collision
  int pad;
  unsigned long long step;       // collision counter (Philox)
  double epot;           // last potential energy (calc_epot substeps)
  int verlet_rebuilds;
  int pad2;
  unsigned long long md_step;    // MD substeps so far (Philox counter of the MD thermostat)
};

// Single-precision constants of one replica for the current collision,
// written once per collision by k_mono_prep (after recentring is known) so
// the FP32 kernels' threads never convert from double.
struct FrameF {
  float L[3];
  float half[3];
  float shear;
  float shearLy;        // shear * Ly: velocity jump across the y face
  float delrx;
  float shift[3];
  float com[3];
  float comv[3];
  float h;
  float kT;
  float solvent_mass;
  float rot_c;
  float rot_s;
  int Li[3];
  int recentre;
  int shear_on;
  int pad[2];
};

// Work tiles: a contiguous range within one replica.
struct Tile {
  int rep;
  int begin;
  int end;
  int pad;
};

struct ErrorState {
  uint32_t word;
  uint32_t info[3];
};

// Per-tile partial sums for the solvent temperature (MPC.cpp:384-418).
struct TempPartial {
  double ekin;
  unsigned filled;
  unsigned pad;
};

}  // namespace smpc
