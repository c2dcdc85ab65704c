// One libsmpc device context per reference Box, shared by the GPU MPC solvent
// (MPC.h in this directory) and the GPU velocity-Verlet integrator
// (Thermostat_GPU.h): MPC collisions change monomer velocities and MD moves
// the monomers, so both act on one device copy of Box::Molecules
// (star-polymers/lib/Box.h:50).
//
// Who owns the monomer state:
//   - with a Thermostat_GPU on the box, the device copy is the live one; the
//     host Box::Molecules is refreshed by Thermostat_GPU::propagate(true),
//     the output steps of the driver loop (star-polymers.cpp:466-519);
//   - without one (CPU thermostat), the host copy is the live one; every
//     collision uploads it and writes the collided state back.
// The context is created at the first step or propagate, when the solvent and
// the molecules are both known (the driver adds the star after constructing
// MPC, star-polymers.cpp:354-370).
#ifndef SMPC_DROPIN_BOX_H_
#define SMPC_DROPIN_BOX_H_

#include <string>
#include <vector>

#include "smpc.h"

class Box;

namespace smpc_dropin {

struct BoxContext {
  smpc_ctx* ctx = nullptr;
  int users = 0;
  // solvent, registered by the MPC constructor (MPC.cpp:10-32)
  bool has_solvent = false;
  double kT = 1.0;
  double shear = 0.0;
  unsigned step_update = 1;
  unsigned n_fluid = 0;
  bool angular_momentum = false;  // MPC(..., angular_mom)
  // integrator, registered by the Thermostat_GPU, AndersenStochastic or
  // Lowe_Andersen constructor (the thermostat kind, its frequency, radius
  // and temperature)
  bool has_md = false;
  double md_dt = 0.01;
  int md_thermostat = SMPC_MDTHERMO_NONE;
  double andersen_nu = 0.0;
  double lowe_radius = 0.0;
  double md_kT = 0.0;  // the thermostat's temperature (> 0), used when there is no solvent
  // device holds the newer monomer state than Box::Molecules
  bool mono_on_device = false;
  bool md_ready = false;
  unsigned n_mono = 0;
};

BoxContext& attach(Box& box);
void detach(Box& box);
BoxContext& find(Box& box);

// Creates the context (first call) and uploads the molecules and their bonds;
// the solvent is uploaded by its owner (MPC::step).
smpc_ctx* ensure(Box& box);

// One velocity-Verlet step of every monomer on the device (the device
// context is created and the MD initialised at the first call); with
// calc_epot the box's monomers, forces and Molecules[0].Epot (the sum over
// all molecules, which Box::print_Epot adds up) are refreshed on the host.
void md_step(Box& box, bool calc_epot);

// Host <-> device copies of the monomer positions and velocities, in
// Box::Molecules order (molecule by molecule, monomer by monomer).
void upload_monomer_state(Box& box);
void download_monomer_state(Box& box, bool with_force);

// Prints the context's last error with `what`, then raises SIGSEGV for device
// cell-range errors (the reference's reaction, MPC.cpp:216-218, 231-233) or
// aborts for anything else.
[[noreturn]] void fail(smpc_ctx* ctx, const char* what, int rc);
void check(smpc_ctx* ctx, const char* what, int rc);
// Reads and clears the device error word; cell-range errors raise SIGSEGV.
void check_device(smpc_ctx* ctx, const char* what);

}  // namespace smpc_dropin

#endif  // SMPC_DROPIN_BOX_H_
