/*
 * smpc.h -- C ABI of the GB300 (sm_103a) coupled MD/MPC step for
 * StarPolymersMD-style systems: star polymers in an SRD/MPC solvent with
 * Lees-Edwards shear. Plain pointers and sizes only; every call returns 0 on
 * success or a positive SMPC_E* code (smpc_last_error() gives the message).
 * Nothing throws across this boundary. One context drives one GPU stream and
 * is not re-entrant; calls are asynchronous except the get/observable calls.
 *
 * A context holds one or many independent replicas (boxes). The reference
 * interfaces each entry point replaces are cited per function; the reference
 * binds them through its C++ classes; the adapter classes (MPC,
 * AndersenStochastic, Lowe_Andersen, Thermostat_GPU over this ABI) are in
 * starpolymersmd_gb300/dropin/.
 */
#ifndef SMPC_H
#define SMPC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SMPC_ABI_VERSION 1

/* return codes */
enum {
  SMPC_OK = 0,
  SMPC_E_ARG = 1,         /* invalid argument */
  SMPC_E_CUDA = 2,        /* CUDA runtime failure */
  SMPC_E_DEVICE = 3,      /* a kernel raised the device error word (see smpc_error_word) */
  SMPC_E_STATE = 4,       /* call not valid in the current state */
  SMPC_E_UNSUPPORTED = 5  /* configuration outside what this build implements */
};

/* device error word bits (smpc_error_word) */
enum {
  SMPC_ERR_FLUID_CELL = 1,    /* solvent cell index out of range (MPC.cpp:211-219) */
  SMPC_ERR_MONO_CELL = 2,     /* monomer cell index out of range (MPC.cpp:227-234) */
  SMPC_ERR_NEIGHBOR_OVF = 4,  /* Verlet list capacity exceeded */
  SMPC_ERR_NONFINITE = 8,     /* non-finite velocity after a collision */
  SMPC_ERR_GAMMA_ITERS = 32,  /* gamma sampler iteration limit */
  SMPC_ERR_FENE = 64,         /* FENE bond at or beyond R0 (Potentials.h:29,50) */
  SMPC_ERR_KEY_MISMATCH = 128, /* internal consistency check of the collide kernel */
  SMPC_ERR_FIXPOINT = 256      /* FP32 path: a particle's m v (or m |v|^2 / 256) reached the
                                  range of the exact fixed-point cell sums, |.| < 4095 */
};

enum { SMPC_FP64 = 0, SMPC_FP32 = 1 };
enum { SMPC_RNG_INJECT = 0, SMPC_RNG_PHILOX = 1 };
enum { SMPC_POT_REF4824 = 0, SMPC_POT_LJ126 = 1 };
enum { SMPC_MONOBIN_REFERENCE = 0, SMPC_MONOBIN_WRAPPED = 1 };
enum { SMPC_DELRX_REFERENCE = 0, SMPC_DELRX_PHYSICAL = 1 };
/* MD thermostats. NONE: Thermostat_None (Thermostat_None.cpp:21-38), the
 * integrator of MPC runs. ANDERSEN: AndersenStochastic (Andersen_stochastic.cpp:
 * 30-59): after each substep every bead, with probability andersen_nu * md_dt,
 * gets new velocity components from N(0, sqrt(kT / m)); draws from Philox on
 * the replica's seed (the reference draws from its global Rand stream), or the
 * resets come from the host (smpc_stage_andersen). */
/* LOWE_ANDERSEN: Lowe_Andersen (Lowe_Andersen.cpp:46-88; the reference's
 * class declares propagate_gaussian without defining it, so its drivers cannot
 * construct it): after the forces of each substep, every Verlet-list pair
 * closer than lowe_radius (at most r_cut) collides with probability
 * nu dt exp(-nu dt) / 2 (nu = andersen_nu), exchanging momentum along its
 * axis with a relative velocity drawn from N(0, sqrt(kT / mu)); collisions in
 * the order beads ascending, partners ascending, with Philox draws; one-star
 * replicas only (SMPC_E_UNSUPPORTED for periodic ones). */
enum { SMPC_MDTHERMO_NONE = 0, SMPC_MDTHERMO_ANDERSEN = 1, SMPC_MDTHERMO_LOWE_ANDERSEN = 2 };
/* Replica flags. SMPC_REPLICA_PERIODIC_MD: the box's monomers (any number of
 * stars) interact through the Lees-Edwards minimum image and are kept in the
 * primary box, with Verlet lists on a periodic cell grid and a rebuild
 * criterion that includes the change of delrx; no recentring (mol0_size only
 * names the default molecule 0). MD substep k of a call (k = 0, 1, ...) uses
 * the delrx that k + 1 further MPC::step(t, h) calls will give (MPC.cpp:117-118).
 * Needs mono_bin = SMPC_MONOBIN_WRAPPED and every L >= 3 r_verlet. The
 * reference integrates one star without periodic images (Box.cpp:105-180). */
enum { SMPC_REPLICA_PERIODIC_MD = 1 };

/* One independent box (MPC + Box + Thermostat_None of the reference). */
typedef struct {
  int L[3];               /* box edge in MPC cells (Box.cpp:14-19; odd L is allowed here) */
  int n_fluid;            /* solvent particles (MPC.cpp:17: N_c * cells) */
  int n_mono;             /* monomers of all molecules of this box */
  int mol0_size;          /* monomers of molecule 0, the recentring reference (MPC.cpp:175-176) */
  double kT;              /* MPC temperature (MPC.cpp:12) */
  double shear;           /* Lees-Edwards shear rate (MPC.cpp:13) */
  double h;               /* collision time step: streaming time of MPC::step(t, h) */
  double md_dt;           /* velocity-Verlet step (Thermostat_None) */
  double lambda;          /* BB attraction (Box.cpp:7) */
  double r_cut;           /* Verlet cut-off (Box.cpp:8) */
  double r_verlet;        /* Verlet radius (Box.cpp:9) */
  double solvent_mass;    /* 1.0 in the reference (MPC.cpp:30) */
  uint64_t seed;          /* Philox key of this box */
  int potential;          /* SMPC_POT_* */
  int flags;              /* SMPC_REPLICA_* bits */
} smpc_replica_desc;

typedef struct {
  int precision;          /* SMPC_FP64 (reference parity) or SMPC_FP32 (fast path) */
  int rng;                /* SMPC_RNG_INJECT or SMPC_RNG_PHILOX */
  int mono_bin;           /* SMPC_MONOBIN_*: reference bins monomers unwrapped (MPC.cpp:223-225) */
  int delrx_mode;         /* SMPC_DELRX_*: reference advances delrx by shear*Ly*dt per MD step */
  int step_update;        /* collide when t % step_update == 0 (MPC.cpp:119); MD substeps per cycle */
  int max_neighbors;      /* Verlet list capacity per monomer (0: default 192) */
  int strict_cells;       /* 1: reference cell formula + range error; 0: clamp into the box */
  int device;             /* CUDA device ordinal */
  int angular_momentum;   /* 1: angular-momentum-conserving collision in cells of more than two
                             particles (MPC.cpp:260-269, 324-374; MPC(..., angular_mom)) */
  int md_thermostat;      /* SMPC_MDTHERMO_*: thermostat of the MD substeps (MPC-off runs) */
  double andersen_nu;     /* collision frequency of SMPC_MDTHERMO_ANDERSEN and _LOWE_ANDERSEN */
  double lowe_radius;     /* interaction radius of SMPC_MDTHERMO_LOWE_ANDERSEN */
} smpc_options;

/* Draws injected for one collision of every replica (reference parity):
 * shift[3*n_rep] (grid shift as constructed at MPC.cpp:123), and per global
 * cell (replicas concatenated in order, cells in MPC::sort order) the gamma
 * variate Gamma(1.5(n-1), kT) for cells with n >= 2 and the raw uniforms of
 * phi = 2 pi u and theta = 2(u - 1/2) (MPC.cpp:244-245, 289). */
typedef struct {
  const double* shift;
  const double* gamma;
  const double* u_phi;
  const double* u_theta;
} smpc_inject;

typedef struct smpc_ctx smpc_ctx;

/* Replaces the MPC / Box / Thermostat_None constructors
 * (MPC.cpp:10-32, Box.cpp:4-27, Thermostat_None.cpp:5-12): allocates device
 * state for n_rep boxes. */
int smpc_create(const smpc_replica_desc* reps, int n_rep, const smpc_options* opt,
                smpc_ctx** out);
void smpc_destroy(smpc_ctx* ctx);
const char* smpc_last_error(const smpc_ctx* ctx);
int smpc_n_cells(const smpc_ctx* ctx, int rep);

/* MPC::initialize / Fluid vector (MPC.h:43, MPC.cpp:34-55): x,y,z interleaved. */
int smpc_set_fluid(smpc_ctx* ctx, int rep, const double* pos, const double* vel);
/* MPC::print_fluid_complete read-out (MPC.cpp:570-579). */
int smpc_get_fluid(smpc_ctx* ctx, int rep, double* pos, double* vel);
/* Box::Molecules state (Box.h:50, Particle.h:48-82). */
int smpc_set_monomers(smpc_ctx* ctx, int rep, const double* pos, const double* vel,
                      const double* force, const double* mass, const int* amphi,
                      const int* anchor);
int smpc_get_monomers(smpc_ctx* ctx, int rep, double* pos, double* vel, double* force);
/* MDParticle::Neighbors, directed (Particle.h:57, Molecule.cpp:146-157). */
int smpc_set_bonds(smpc_ctx* ctx, int rep, int n_bond, const int* src, const int* dst);
/* Thermostat_None constructor body: Verlet lists + forces (Thermostat_None.cpp:9-11). */
int smpc_init_md(smpc_ctx* ctx);

/* n x Thermostat_None::propagate(calc_epot) for every replica
 * (Thermostat_None.cpp:21-38); the potential energy of the last substep is
 * kept when calc_epot != 0 (Box::print_Epot, Box.cpp:605-613). */
int smpc_md_substeps(smpc_ctx* ctx, int n, int calc_epot);
/* The Andersen resets of replica rep's next n_steps MD substeps, given by the
 * host in place of the device's draws: in substep s (0-based) of the next
 * smpc_md_substeps call (which must have n == n_steps), replica-local monomer
 * mono[e] gets the velocity vel[3e .. 3e+2] after the second half kick, for
 * e in [step_start[s], step_start[s + 1]). The reference's loop of
 * AndersenStochastic::propagate (Andersen_stochastic.cpp:49-58: one
 * Rand::real_uniform() per monomer, three Rand::real_normal(0, sigma) when it
 * is below nu * dt) runs on the host, so a drop-in replays the reference's
 * global Rand stream exactly. Needs SMPC_MDTHERMO_ANDERSEN; not for periodic
 * replicas (SMPC_E_UNSUPPORTED). Replicas without staged resets draw. */
int smpc_stage_andersen(smpc_ctx* ctx, int rep, int n_steps, const int* step_start,
                        const int* mono, const double* vel);
/* MPC::step(t, dt) for every replica (MPC.cpp:116-142): delrx advance on every
 * call, a collision when t % step_update == 0. inj may be NULL only in
 * Philox mode. */
int smpc_mpc_step(smpc_ctx* ctx, long t, double dt, const smpc_inject* inj);
/* MPC::step in two phases, for drivers that draw the collision's random
 * numbers themselves in the reference's order (grid shift before binning,
 * then per cell gamma, phi, theta -- MPC.cpp:123, 244-245, 289), e.g. from
 * the reference's own Rand stream:
 *   smpc_mpc_bin: delrx advance; on a collision step (*collide_now = 1)
 *     recentring, streaming, the grid shift (shift[3*n_rep], or NULL for the
 *     Philox shift) and the counting sort; smpc_cell_counts then gives the
 *     occupancies that decide which cells draw a gamma variate;
 *   smpc_mpc_collide: the per-cell collisions with injected draws (inj) or
 *     Philox draws (inj == NULL), and the unshift. */
int smpc_mpc_bin(smpc_ctx* ctx, long t, double dt, const double* shift, int* collide_now);
int smpc_mpc_collide(smpc_ctx* ctx, const smpc_inject* inj);
/* n fused cycles of (step_update MD substeps + one collision) with Philox
 * draws, launched as a captured CUDA graph. */
int smpc_cycles(smpc_ctx* ctx, int n);

/* Same cycles launched on the context stream with CUDA events around every
 * phase (phase_ms[8]: MD substeps, cycle begin, monomer prep, solvent bin,
 * scan, perm, collide, cycle end; summed over the n cycles) and the total
 * elapsed time from the first to the last event. */
int smpc_cycles_profiled(smpc_ctx* ctx, int n, double* phase_ms, int n_phases, double* total_ms);
/* Launch-shape variants of the FP32 fast-path kernels (solvent binning,
 * collide, MD substeps); index 0 is the default. Changing them re-captures
 * the cycle graph. FP64 contexts of few replicas run each replica's MD on a
 * cluster of SMs; md = 1 keeps one CTA per replica there instead. */
int smpc_set_variants(smpc_ctx* ctx, int bin, int collide, int md);
int smpc_get_variants(const smpc_ctx* ctx, int* bin, int* collide, int* md);
/* Launch-shape variant of the periodic-MD kernels of FP32 contexts (lanes per
 * bead of the force kernel, grid of the list builder; index 0 is the
 * default). Each variant sums a bead's forces in its own fixed order. */
int smpc_set_pmd_variant(smpc_ctx* ctx, int pmd);
int smpc_get_pmd_variant(const smpc_ctx* ctx, int* pmd);
/* Times every variant of each fast-path kernel (and, in contexts with periodic
 * boxes, of the periodic MD) over `cycles` cycles of the
 * context's own workload (CUDA events on the context stream), keeps the
 * fastest and writes a JSON report (variant -> ms per cycle, chosen). The
 * state is saved to host memory before the trials (as smpc_checkpoint_save)
 * and restored after them, so the simulation does not advance. */
int smpc_autotune(smpc_ctx* ctx, int cycles, char* report, int report_len);
/* smpc_cycles bracketed by CUDA events on the context stream (ms). */
int smpc_time_cycles(smpc_ctx* ctx, int n, double* total_ms);
/* Solvent initial state generated on the device (MPC::initialize,
 * MPC.cpp:34-55): positions uniform in the box; velocities uniform in
 * [-1/2, 1/2) with SMPC_INIT_REFERENCE_VELOCITIES, else Maxwell-Boltzmann at
 * kT, minus their mean, so the solvent's total momentum is zero as in the
 * reference; SMPC_INIT_SHEAR_PROFILE then adds the steady Lees-Edwards flow
 * shear * y to v_x (a long sheared run's state, instead of a fluid at rest). */
enum { SMPC_INIT_REFERENCE_VELOCITIES = 1, SMPC_INIT_SHEAR_PROFILE = 2 };
int smpc_init_solvent(smpc_ctx* ctx, int rep, uint64_t seed, int flags);

/* Observables. */
int smpc_temperature(smpc_ctx* ctx, int rep, double* out);   /* MPC.cpp:405-409 */
int smpc_epot(smpc_ctx* ctx, int rep, double* out);          /* sum of Molecule::Epot */
/* Temperature of every replica (out[n_rep]) from one kernel launch. */
int smpc_temperature_all(smpc_ctx* ctx, double* out);
/* smpc_temperature_all without allocating anything, device or host (no
 * counterpart in the reference, whose temperature is a host loop): the
 * per-tile partial sums and per-replica results live in one static device
 * array of 544 KB, at most 32768 temperature tiles (512 cells each, 16.7 M
 * cells) and 4096 replicas per context; larger contexts get
 * SMPC_E_UNSUPPORTED. For callers that cannot allocate mid-run. The first call
 * on a device looks up the array's address (set-up); make it before any
 * stream capture. The array is shared by every context of the process on that
 * device: calls that overlap in time race on it. */
int smpc_temperature_all_noalloc(smpc_ctx* ctx, double* out);
/* Monomer positions/velocities of all replicas (concatenated, x,y,z
 * interleaved): the Box::Molecules state a host-side driver reads and writes
 * between steps (star-polymers.cpp:466-519). Masses and types are kept. The
 * stored forces are kept too (velocity Verlet carries them into the next
 * substep's first half kick, Thermostat_None.cpp:21-27): after placing a
 * different configuration, smpc_init_md recomputes them. Periodic replicas
 * rebuild their Verlet lists at the next substep. */
int smpc_set_monomer_state_all(smpc_ctx* ctx, const double* pos, const double* vel);
int smpc_get_monomer_state_all(smpc_ctx* ctx, double* pos, double* vel, double* force);
/* One call per output step of a host-side driver (star-polymers.cpp:466-534):
 * smpc_set_monomer_state_all(pos_in, vel_in) when pos_in is given, n fused
 * cycles (smpc_cycles), smpc_get_monomer_state_all(pos_out, vel_out) when
 * pos_out is given and smpc_molecule_observables_all(obs_out) when obs_out is
 * given, queued on the context's stream with one synchronisation at the end
 * (copies from and to pinned buffers overlap nothing else but skip the host
 * round trips between the parts). pos_in and pos_out may be the same array. */
int smpc_cycles_io(smpc_ctx* ctx, int n, const double* pos_in, const double* vel_in,
                   double* pos_out, double* vel_out, double* obs_out);
int smpc_delrx(smpc_ctx* ctx, int rep, double* out);
int smpc_set_delrx(smpc_ctx* ctx, int rep, double delrx);
/* Cell occupancies of the last collision: MPCCellList sizes and
 * MPCCellListFluidParticles (MPC.h:40-41). */
int smpc_cell_counts(smpc_ctx* ctx, int rep, unsigned* total, unsigned* fluid);
/* Cell of every solvent particle (fluid_cell[n_fluid], by particle id) and of
 * every monomer (mono_cell[n_mono], -1 if not binned) at the last collision:
 * MPCParticle::CellIndex as MPC::sort set it (MPC.cpp:209, 224), from which a
 * host-side driver rebuilds MPCCellList (MPC.h:40) for its per-cell getters
 * (calculateFluidVelocity, calculateEkinInCell, print_fluid; MPC.cpp:335-418,
 * 533-568). SMPC_E_STATE after a solvent upload or a binning without its
 * collision. Either pointer may be NULL. */
int smpc_cell_members(smpc_ctx* ctx, int rep, int* fluid_cell, int* mono_cell);
int smpc_set_collision_counter(smpc_ctx* ctx, uint64_t counter);

/* Molecules of a replica (Box::Molecules, Box.h:50): mol_start[n_mol + 1]
 * monomer offsets within the replica, from 0 to n_mono, every molecule
 * non-empty. Default: molecule 0 = the first mol0_size monomers, the rest one
 * more molecule. Used by the observables below. */
int smpc_set_molecules(smpc_ctx* ctx, int rep, int n_mol, const int* mol_start);
/* Output-step observables of every replica from one launch, FP64
 * (star-polymers.cpp:467-473), out[SMPC_OBS_PER_REP * n_rep]; per replica, in
 * each molecule's centre-of-mass frame (Box::center_of_mass_reference_frame,
 * Box.cpp:81-102): [0] R_g and [1..9] gyration tensor G (row-major), both
 * averaged over molecules (Box::calculate_gyration_tensor, Box.cpp:330-353);
 * [10..12] rotation frequency averaged over molecules
 * (Box::calculate_rotation_frequency, Box.cpp:355-379); [13] kinetic energy
 * (Box::calculate_ekin, Box.cpp:288-294); [14] the temperature
 * 2 E / (3 (N - 1)) (Box::print_Ekin_and_Temperature, Box.cpp:635-646);
 * [15] the number of molecules. */
#define SMPC_OBS_PER_REP 16
int smpc_molecule_observables_all(smpc_ctx* ctx, double* out);
/* VelocityX once over a replica's solvent (Velocity_x.h:76-100, applied as
 * star-polymers.cpp:483 does): velocity relative to molecule 0's mean
 * velocity, binned by floor(p / width) of the Lees-Edwards-wrapped position
 * relative to molecule 0's centre (MPC::wrap(pos, vel), MPC.cpp:492-495),
 * along x (x_out) and along y (y_out). Bin k of an axis of length L sits at
 * out[3 (k - floor(-L / (2 width)))] = (sum v_x, sum v_y, count); an axis needs
 * floor(L / (2 width)) - floor(-L / (2 width)) + 1 bins (SMPC_E_ARG otherwise). */
int smpc_velocity_profile(smpc_ctx* ctx, int rep, double width, double* x_out, int n_x,
                          double* y_out, int n_y);
int smpc_verlet_rebuilds(smpc_ctx* ctx, int rep, int* out);

/* Device error word (0 = clean) and its first offender; clears it. */
int smpc_error_word(smpc_ctx* ctx, unsigned* word, unsigned* info3);
int smpc_synchronize(smpc_ctx* ctx);

/* Solvent analyses (the reference's Analysis functors, sums on the device).
 * smpc_fourier_modes: Fourier_Autocorr::operator() (Fourier_Autocorr.h) for one
 *   sample: for k = (2 pi / box_length) e_j, j = x, y, z, the transverse mode
 *   sum_i v_i exp(i k . r_i) / N with its j component removed; out18 =
 *   3 modes x 3 components x (re, im).
 * smpc_vacf_*: Vel_Autocorr_Fluid (Vel_Autocorr_Fluid.h) over solvent
 *   particles 0..n_particles-1 of one replica: a window of `entries`
 *   velocity samples (one per smpc_vacf_sample); once it is full, every
 *   sample adds sum_i v_i(oldest) . v_i(oldest + j) to lag_sums[j]. The
 *   reference's average is lag_sums[j] / calculations / n_particles. */
int smpc_fourier_modes(smpc_ctx* ctx, int rep, double box_length, double* out18);
/* Pressure tensor of every replica (no reference counterpart): out[12 r + k],
 * k = 0..5 the kinetic part (1/V) sum m u u^T over solvent and monomers with
 * the peculiar velocity u = v - shear y e_x, k = 6..11 the monomers' pair and
 * FENE virial (1/V) sum over pairs r_ij F_ij^T; components xx yy zz xy xz yz.
 * The SRD collision's momentum transfer is not included. */
int smpc_pressure_tensor_all(smpc_ctx* ctx, double* out);
int smpc_vacf_start(smpc_ctx* ctx, int rep, int n_particles, int entries);
int smpc_vacf_sample(smpc_ctx* ctx);
int smpc_vacf_result(smpc_ctx* ctx, double* lag_sums, uint64_t* calculations);

/* Checkpoint / restart. Replaces the reference's restart files -- the fluid
 * as "%f" text (MPC::print_fluid_complete, MPC.cpp:570-579, read back by
 * MPC::initialize(filename, Box_old), MPC.cpp:57-113) and the stars as PDB
 * with velocities at %7.3f (Box::print_PDB_with_velocity, Box.cpp:563-602,
 * read back by Molecule::star_from_file, Molecule.cpp:178-224), after which
 * the reference re-seeds its random stream. A checkpoint here holds the
 * context's full state at its own precision: solvent records, monomer state
 * with forces and Verlet lists, every replica's delrx and Philox collision
 * counter, bonds, molecules and the periodic-MD bookkeeping. Loading it into
 * a context created with the same replicas and options continues the run bit
 * for bit. Call between steps (not between smpc_mpc_bin and
 * smpc_mpc_collide). A load that fails validation (other replicas, options or
 * format) leaves the context unchanged; a truncated stream leaves it undefined. */
int smpc_checkpoint_size(smpc_ctx* ctx, uint64_t* bytes);
int smpc_checkpoint_save(smpc_ctx* ctx, void* buf, uint64_t capacity);
int smpc_checkpoint_load(smpc_ctx* ctx, const void* buf, uint64_t length);
int smpc_checkpoint_write(smpc_ctx* ctx, const char* path);
int smpc_checkpoint_read(smpc_ctx* ctx, const char* path);

#ifdef __cplusplus
}
#endif
#endif
