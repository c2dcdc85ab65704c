/*
 * smpc_oracle.h -- CPU restatement (plain C, FP64) of the StarPolymersMD
 * coupled MD/MPC step. TEST INFRASTRUCTURE ONLY: the parity tests, smoke()
 * and bench.py's CPU-baseline leg are the only callers; the product never
 * links or calls it.
 *
 * It follows the reference's arithmetic order operation by operation so that
 * it reproduces the reference's results bit for bit on identical inputs:
 *   MPC::step / check_bounds / streaming / sort / calculateCMV / thermostat /
 *   collide / shiftParticles / LEBC / wrap  (star-polymers/lib/Hydrodynamics/MPC.cpp)
 *   Thermostat_None::propagate              (star-polymers/lib/Thermostats/Thermostat_None.cpp:21-38)
 *   Box::update_VerletLists / check_VerletLists / calculate_forces_verlet
 *                                           (star-polymers/lib/Box.cpp:105-286)
 *   FENE / 48-24 pair potentials            (star-polymers/lib/Molecules/Potentials.h:14-120)
 * Parity is pinned against the reference compiled from its own sources
 * (oracle/refbuild) through the fixtures in tests/golden.
 *
 * Random numbers come from one of two sources:
 *   ORC_RNG_INJECT -- per-collision arrays (grid shift, per-cell gamma variate,
 *                     per-cell raw uniforms for phi and theta) recorded from
 *                     the reference's own mt19937_64 stream;
 *   ORC_RNG_PHILOX -- the project's counter-based stream (Philox4x32-10 plus
 *                     Marsaglia-Tsang gamma), restated here independently of
 *                     the CUDA implementation (layout in smpc_oracle.c).
 */
#ifndef SMPC_ORACLE_H
#define SMPC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_RNG_INJECT = 0, ORC_RNG_PHILOX = 1 };
enum { ORC_POT_REF4824 = 0, ORC_POT_LJ126 = 1 };

/* Error codes (bit flags) mirroring the reference's fatal paths. */
enum {
  ORC_ERR_FLUID_CELL = 1,   /* MPC.cpp:211-219: fluid CellIndex out of range */
  ORC_ERR_MONO_CELL = 2,    /* MPC.cpp:227-234: monomer CellIndex out of range */
  ORC_ERR_VERLET_CELL = 4,  /* Box.cpp:132-142: monomer outside the Verlet grid */
  ORC_ERR_ALLOC = 8,
  ORC_ERR_INJECT = 16       /* inject mode without injected draws */
};

typedef struct {
  int L[3];              /* box edge in MPC cells (callers bump odd L like Box.cpp:14-16) */
  double kT;             /* MPC temperature (MPC.cpp:12) */
  double shear;          /* Lees-Edwards shear rate (MPC.cpp:13) */
  unsigned step_update;  /* collide when t % step_update == 0 (MPC.cpp:119) */
  int angular_momentum;  /* MPC.cpp:15: angular-momentum-conserving collision */
  double lambda;         /* BB attraction depth (Box.cpp:7) */
  double md_dt;          /* velocity-Verlet step (Thermostat.cpp:3) */
  double r_cut;          /* Verlet cut-off (Box.cpp:8, 1.5) */
  double r_verlet;       /* Verlet radius (Box.cpp:9, 2.0) */
  int potential;         /* ORC_POT_REF4824 (reference) or ORC_POT_LJ126 */
  double delrx_dt_scale; /* 1.0: delrx advances by shear*Ly*dt per call as MPC.cpp:117;
                            1/step_update: physical advance */
  int mono_wrap;         /* 0: monomers binned unwrapped (MPC.cpp:223-225);
                            1: binned at their Lees-Edwards periodic image */
} orc_params;

typedef struct smpc_orc smpc_orc;

smpc_orc* orc_create(const orc_params* p, long n_fluid, int n_mono, int n_mol,
                     const int* mol_start /* n_mol+1 monomer offsets */);
void orc_destroy(smpc_orc* o);
int orc_error(const smpc_orc* o);
void orc_clear_error(smpc_orc* o);

/* State in/out (x,y,z interleaved per particle). */
void orc_set_fluid(smpc_orc* o, const double* pos, const double* vel);
void orc_get_fluid(const smpc_orc* o, double* pos, double* vel);
void orc_set_monomers(smpc_orc* o, const double* pos, const double* vel, const double* force,
                      const double* mass, const int* amphi, const int* anchor);
void orc_get_monomers(const smpc_orc* o, double* pos, double* vel, double* force);
/* Directed FENE bonds (MDParticle::Neighbors order, source-major). */
void orc_set_bonds(smpc_orc* o, int n_bond, const int* src, const int* dst);
/* Thermostat_None constructor: Verlet lists + forces (Thermostat_None.cpp:5-12). */
void orc_init_md(smpc_orc* o);
/* Periodic MD of many molecules (call before orc_init_md; needs mono_wrap = 1):
 * every pair and bond distance is the Lees-Edwards minimum image, monomers are
 * wrapped into the primary box with the v_x jump, no recentring; MD step t uses
 * the delrx the next MPC::step(t, h) call gives. */
void orc_set_periodic_md(smpc_orc* o, double h);
/* Andersen stochastic thermostat after every MD step (MPC-off runs). */
void orc_set_andersen(smpc_orc* o, double nu, uint64_t seed);
/* Lowe-Andersen pair thermostat after the forces of every MD step (MPC-off
 * runs; non-periodic boxes). */
void orc_set_lowe_andersen(smpc_orc* o, double nu, double radius, uint64_t seed);
/* The next MD step's Andersen resets given explicitly (monomer idx[k] gets
 * vel[3k..3k+2] after the second half kick) instead of drawn. */
void orc_stage_andersen(smpc_orc* o, int n, const int* idx, const double* vel);
/* Periodic forces at the current positions and delrx into out[3 n_mono]: by
 * the cell grid that large boxes use (force_grid = 1) or by the loop over all
 * monomers (0). The state is not changed. */
void orc_periodic_forces(smpc_orc* o, int force_grid, double* out);

double orc_delrx(const smpc_orc* o);
void orc_set_delrx(smpc_orc* o, double d);

/* RNG sources. Inject arrays are borrowed until the next orc_mpc_step. */
void orc_set_inject(smpc_orc* o, const double* shift3, const double* gamma,
                    const double* u_phi, const double* u_theta);
void orc_set_philox(smpc_orc* o, uint64_t seed, uint64_t collision_counter);
uint64_t orc_collision_counter(const smpc_orc* o);

/* MPC::step(t, dt) (MPC.cpp:116-142). */
void orc_mpc_step(smpc_orc* o, long t, double dt);
/* Thermostat_None::propagate(calc_epot) (Thermostat_None.cpp:21-38). */
void orc_propagate(smpc_orc* o, int calc_epot);
/* n iterations of the star-polymers.cpp loop body: propagate then MPC::step. */
void orc_run(smpc_orc* o, long t0, long n, double mpc_dt, int with_md);

/* Observables. */
double orc_temperature(smpc_orc* o);      /* MPC::calculateCurrentTemperature (MPC.cpp:405-409) */
double orc_epot(const smpc_orc* o);       /* sum of Molecule::Epot */
unsigned orc_n_cells(const smpc_orc* o);
void orc_cell_counts(const smpc_orc* o, unsigned* total, unsigned* fluid);
int orc_verlet_rebuilds(const smpc_orc* o);
/* Reference Philox4x32-10 block (for known-answer tests). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* The project's gamma sampler on the Philox stream (shape a >= 1, scale 1). */
double orc_philox_gamma(uint64_t seed, uint64_t step, uint32_t cell, double shape);

/* Collision draws (rotation axis and gamma sampler, not the grid shift) from
 * the FP32 path's 23-bit uniforms (w >> 9) 2^-23 + 2^-24 of the same Philox
 * words, so the oracle consumes exactly the values the FP32 kernels do. */
void orc_set_f32_uniforms(smpc_orc* o, int on);
/* Cells of the last collision per solvent particle and monomer (-1: none). */
void orc_cell_members(const smpc_orc* o, int* fluid_cell, int* mono_cell);

#ifdef __cplusplus
}
#endif
#endif
