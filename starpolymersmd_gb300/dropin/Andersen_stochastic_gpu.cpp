// The reference's AndersenStochastic (star-polymers/lib/Thermostats/
// Andersen_stochastic.h, unchanged) with its MD on the GPU: this file replaces
// Andersen_stochastic.cpp when a driver is built against the drop-ins, so the
// MPC-off branch of star-polymers.cpp:387 (AndersenStochastic{box, StepSize,
// Temperature, 0.1}) runs through libsmpc.
//
// The velocity resets keep the reference's random stream: propagate() makes
// the draws of Andersen_stochastic.cpp:49-58 on the host, from the reference's
// own Rand, in the same order (one Rand::real_uniform() per monomer in
// Box::Molecules order; three Rand::real_normal(0, sigma) for a monomer whose
// uniform is below nu dt), and hands the resulting velocities to the device
// (smpc_stage_andersen), which sets them after the second half kick. The
// draws do not depend on the state, so drawing before the device step leaves
// the stream and the results unchanged.
//
// The reference class declares no destructor, so the box's device context is
// released with the process (or by the GPU MPC, if it is the last user).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Andersen_stochastic.h"
#include "Rand.h"
#include "smpc.h"
#include "smpc_box.h"

const std::string AndersenStochastic::Name = "Andersen stochastic";

// Andersen_stochastic.cpp:11-22: the host builds the Verlet lists and forces
// once, so the Box holds valid forces after construction; the device rebuilds
// both at the first propagate.
AndersenStochastic::AndersenStochastic(Box& box, double dt, double T, double nu, bool gaussian)
    : Thermostat(box, dt), TargetTemperature(T), Nu(nu), Sigma(std::sqrt(T)) {
  if (gaussian) {
    std::fprintf(stderr,
                 "AndersenStochastic (GPU): Gaussian chains (harmonic bonds, Box.cpp:677-706) "
                 "are not implemented on the GPU\n");
    std::abort();
  }
  smpc_dropin::BoxContext& bc = smpc_dropin::attach(SimBox);
  bc.has_md = true;
  bc.md_dt = dt;
  bc.md_thermostat = SMPC_MDTHERMO_ANDERSEN;
  bc.andersen_nu = nu;
  bc.md_kT = T;
  update_temp();
  dtime(dt);
  SimBox.update_VerletLists();
  SimBox.calculate_forces_verlet();
}

void AndersenStochastic::update_temp() {}

void AndersenStochastic::dtime(double& dt) {
  smpc_dropin::BoxContext& bc = smpc_dropin::find(SimBox);
  if (bc.ctx && dt != bc.md_dt) {
    std::fprintf(stderr,
                 "AndersenStochastic (GPU): the time step is fixed once the GPU context exists\n");
    std::abort();
  }
  Thermostat::dtime(dt);
  DeltaTHalf = DeltaT * 0.50;
  bc.md_dt = dt;
}

// Andersen_stochastic.cpp:30-59: half kick, drift, Verlet check, forces, half
// kick on the device; the resets drawn here from the reference's Rand.
void AndersenStochastic::propagate(bool calc_epot) {
  std::vector<int> mono, start{0, 0};
  std::vector<double> vel;
  int k = 0;
  for (auto& mol : SimBox.Molecules)
    for (auto& m : mol.Monomers) {
      if (Rand::real_uniform() < Nu * DeltaT) {
        mono.push_back(k);
        for (unsigned i = 0; i < 3; i++)
          vel.push_back(m.Mass == 1.0 ? Rand::real_normal(0.0, Sigma)
                                      : Rand::real_normal(0.0, Sigma / std::sqrt(m.Mass)));
      }
      ++k;
    }
  start[1] = static_cast<int>(mono.size());
  smpc_ctx* ctx = smpc_dropin::ensure(SimBox);
  smpc_dropin::check(ctx, "smpc_stage_andersen",
                     smpc_stage_andersen(ctx, 0, 1, start.data(), mono.data(), vel.data()));
  smpc_dropin::md_step(SimBox, calc_epot);
}

void AndersenStochastic::propagate_gaussian(bool) {
  std::fprintf(stderr, "AndersenStochastic::propagate_gaussian is not implemented on the GPU\n");
  std::abort();
}

std::string AndersenStochastic::name() const { return Name; }

std::string AndersenStochastic::info() const {
  return std::string("Thermostat ") + Name + " dtime " + std::to_string(DeltaT);
}
