// GPU velocity-Verlet integrator behind the reference's Thermostat interface
// (Thermostat_GPU.h). Reference behaviour: star-polymers/lib/Thermostats/
// Thermostat_None.cpp (constructor :5-12, propagate :21-38).
#include "Thermostat_GPU.h"

#include <cstdio>
#include <cstdlib>

#include "smpc.h"
#include "smpc_box.h"

const std::string Thermostat_GPU::Name = "GPU";

// Thermostat_None.cpp:5-12: the host builds the Verlet lists and forces once,
// so the Box holds valid forces right after construction as with the CPU
// integrator; the device rebuilds both at the first propagate.
Thermostat_GPU::Thermostat_GPU(Box& box, double dt, bool gaussian) : Thermostat(box, dt) {
  if (gaussian) {
    std::fprintf(stderr,
                 "Thermostat_GPU: Gaussian chains (harmonic bonds, Box.cpp:677-706) are not "
                 "implemented on the GPU\n");
    std::abort();
  }
  smpc_dropin::BoxContext& bc = smpc_dropin::attach(SimBox);
  bc.has_md = true;
  bc.md_dt = dt;
  update_temp();
  dtime(dt);
  SimBox.update_VerletLists();
  SimBox.calculate_forces_verlet();
}

Thermostat_GPU::~Thermostat_GPU() { smpc_dropin::detach(SimBox); }

void Thermostat_GPU::update_temp() {}

void Thermostat_GPU::dtime(double& dt) {
  smpc_dropin::BoxContext& bc = smpc_dropin::find(SimBox);
  if (bc.ctx && dt != bc.md_dt) {
    std::fprintf(stderr, "Thermostat_GPU: the time step is fixed once the GPU context exists\n");
    std::abort();
  }
  Thermostat::dtime(dt);
  DeltaTHalf = DeltaT * 0.50;
  bc.md_dt = dt;
}

// Thermostat_None.cpp:21-38 on the device: half kick, drift, Verlet check and
// rebuild, forces (with the potential energy when calc_epot), half kick.
void Thermostat_GPU::propagate(bool calc_epot) { smpc_dropin::md_step(SimBox, calc_epot); }

void Thermostat_GPU::propagate_gaussian(bool) {
  std::fprintf(stderr, "Thermostat_GPU::propagate_gaussian is not implemented on the GPU\n");
  std::abort();
}

std::string Thermostat_GPU::name() const { return Name; }

std::string Thermostat_GPU::info() const {
  return std::string("Thermostat ") + Name + " dtime " + std::to_string(DeltaT);
}
