// The reference's Lowe_Andersen (star-polymers/lib/Thermostats/Lowe_Andersen.h,
// unchanged) with its MD and pair collisions on the GPU
// (SMPC_MDTHERMO_LOWE_ANDERSEN). The reference's own Lowe_Andersen.cpp
// declares propagate_gaussian in the header without defining it, so no driver
// can construct that class; compiled in its place, this file makes the
// commented-out MPC-off branch of star-polymers.cpp:388
// (Lowe_Andersen{box, StepSize, Temperature, 20., 1.5}) usable.
//
// Differences from the reference, both stated in include/smpc.h: the pair
// draws come from Philox on the device, not from the reference's Rand, and
// the collisions run in the order beads ascending, partners ascending (the
// reference walks each bead's Verlet list in its cell-list order).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "Lowe_Andersen.h"
#include "smpc.h"
#include "smpc_box.h"

const std::string Lowe_Andersen::Name = "Lowe_Andersen";

// Lowe_Andersen.cpp:6-16: the host computes the forces once, so the Box holds
// valid forces after construction; the device rebuilds lists and forces at
// the first propagate.
Lowe_Andersen::Lowe_Andersen(Box& box, double dt, double temp, double nu, double r)
    : Thermostat(box, dt), TargetTemperature(temp), Nu(nu), InteractionRadius{r} {
  smpc_dropin::BoxContext& bc = smpc_dropin::attach(SimBox);
  bc.has_md = true;
  bc.md_dt = dt;
  bc.md_thermostat = SMPC_MDTHERMO_LOWE_ANDERSEN;
  bc.andersen_nu = nu;
  bc.lowe_radius = r;
  bc.md_kT = temp;
  update_temp();
  dtime(dt);
  SimBox.update_VerletLists();
  SimBox.calculate_forces_verlet();
}

void Lowe_Andersen::update_temp() {}

// Lowe_Andersen.cpp:21-26
void Lowe_Andersen::dtime(double& dt) {
  smpc_dropin::BoxContext& bc = smpc_dropin::find(SimBox);
  if (bc.ctx && dt != bc.md_dt) {
    std::fprintf(stderr, "Lowe_Andersen (GPU): the time step is fixed once the GPU context exists\n");
    std::abort();
  }
  Thermostat::dtime(dt);
  DeltaTHalf = DeltaT * 0.5;
  NuDt = Nu * DeltaT * std::exp(-DeltaT * Nu);
  std::cout << "NuDt = " << NuDt << std::endl;
  bc.md_dt = dt;
}

void Lowe_Andersen::collide(Particle&, Particle&) {
  std::fprintf(stderr, "Lowe_Andersen::collide: the pair collisions run on the GPU\n");
  std::abort();
}

// Lowe_Andersen.cpp:46-88 on the device: half kick, drift, Verlet check,
// forces, pair collisions, half kick.
void Lowe_Andersen::propagate(bool calc_epot) { smpc_dropin::md_step(SimBox, calc_epot); }

void Lowe_Andersen::propagate_gaussian(bool) {
  std::fprintf(stderr, "Lowe_Andersen::propagate_gaussian is not implemented\n");
  std::abort();
}

std::string Lowe_Andersen::name() const { return Name; }

// Lowe_Andersen.cpp:90-98
std::string Lowe_Andersen::info() const {
  return std::string("Thermostat ") + Name + " dtime " + std::to_string(DeltaT) + " nu " +
         std::to_string(Nu);
}
