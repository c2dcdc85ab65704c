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
void Thermostat_GPU::propagate(bool calc_epot) {
  smpc_dropin::BoxContext& bc = smpc_dropin::find(SimBox);
  smpc_ctx* ctx = smpc_dropin::ensure(SimBox);
  if (!bc.md_ready) {
    if (!bc.mono_on_device) smpc_dropin::upload_monomer_state(SimBox);
    smpc_dropin::check(ctx, "smpc_init_md", smpc_init_md(ctx));
    bc.md_ready = true;
    bc.mono_on_device = true;
  }
  smpc_dropin::check(ctx, "smpc_md_substeps", smpc_md_substeps(ctx, 1, calc_epot ? 1 : 0));
  if (!calc_epot) return;
  smpc_dropin::check_device(ctx, "Thermostat_GPU::propagate");
  smpc_dropin::download_monomer_state(SimBox, true);
  double epot = 0.;
  smpc_dropin::check(ctx, "smpc_epot", smpc_epot(ctx, 0, &epot));
  // the device sums the potential energy over all molecules; Box::print_Epot
  // (Box.cpp:605-613) reads the sum over Molecules
  for (auto& mol : SimBox.Molecules) mol.Epot = 0.0;
  if (!SimBox.Molecules.empty()) SimBox.Molecules[0].Epot = epot;
}

void Thermostat_GPU::propagate_gaussian(bool) {
  std::fprintf(stderr, "Thermostat_GPU::propagate_gaussian is not implemented on the GPU\n");
  std::abort();
}

std::string Thermostat_GPU::name() const { return Name; }

std::string Thermostat_GPU::info() const {
  return std::string("Thermostat ") + Name + " dtime " + std::to_string(DeltaT);
}
