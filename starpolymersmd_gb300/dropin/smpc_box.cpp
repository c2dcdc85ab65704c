// Shared per-Box device context of the GPU drop-ins (see smpc_box.h).
#include "smpc_box.h"

#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <unordered_map>

#include "Box.h"
#include "Particle.h"

namespace smpc_dropin {

namespace {

std::map<const Box*, BoxContext>& registry() {
  static std::map<const Box*, BoxContext> r;
  return r;
}

int device_ordinal() {
  const char* s = std::getenv("SMPC_DEVICE");
  return s ? std::atoi(s) : 0;
}

unsigned count_monomers(const Box& box) {
  unsigned n = 0;
  for (const auto& mol : box.Molecules) n += static_cast<unsigned>(mol.Monomers.size());
  return n;
}

void flatten(Box& box, std::vector<double>& pos, std::vector<double>& vel,
             std::vector<double>* force) {
  const unsigned n = count_monomers(box);
  pos.resize(3 * static_cast<size_t>(n));
  vel.resize(3 * static_cast<size_t>(n));
  if (force) force->resize(3 * static_cast<size_t>(n));
  size_t k = 0;
  for (const auto& mol : box.Molecules)
    for (const auto& mono : mol.Monomers) {
      for (int d = 0; d < 3; ++d) {
        pos[3 * k + d] = mono.Position(d);
        vel[3 * k + d] = mono.Velocity(d);
        if (force) (*force)[3 * k + d] = mono.Force(d);
      }
      ++k;
    }
}

}  // namespace

BoxContext& attach(Box& box) {
  BoxContext& bc = registry()[&box];
  ++bc.users;
  return bc;
}

BoxContext& find(Box& box) {
  auto it = registry().find(&box);
  if (it == registry().end()) {
    std::fprintf(stderr, "smpc drop-in: box has no GPU context\n");
    std::abort();
  }
  return it->second;
}

void detach(Box& box) {
  auto it = registry().find(&box);
  if (it == registry().end()) return;
  if (--it->second.users > 0) return;
  if (it->second.ctx) smpc_destroy(it->second.ctx);
  registry().erase(it);
}

void fail(smpc_ctx* ctx, const char* what, int rc) {
  std::fprintf(stderr, "smpc drop-in: %s failed (code %d): %s\n", what, rc,
               ctx ? smpc_last_error(ctx) : "no context");
  std::fflush(stderr);
  std::abort();
}

void check(smpc_ctx* ctx, const char* what, int rc) {
  if (rc == SMPC_E_DEVICE) check_device(ctx, what);
  if (rc != SMPC_OK) fail(ctx, what, rc);
}

void check_device(smpc_ctx* ctx, const char* what) {
  unsigned word = 0, info[3] = {0, 0, 0};
  const int rc = smpc_error_word(ctx, &word, info);
  if (rc != SMPC_OK) fail(ctx, "smpc_error_word", rc);
  if (!word) return;
  if (word & (SMPC_ERR_FLUID_CELL | SMPC_ERR_MONO_CELL)) {
    // the reference prints the offender and raises SIGSEGV; drivers install a
    // handler that dumps the configuration (star-polymers.cpp:414-419)
    std::cout << "CellIndex of " << ((word & SMPC_ERR_FLUID_CELL) ? "fluid" : "monomer")
              << " out of range! (device error word " << word << ", particle " << info[0]
              << ", " << what << ")" << std::endl;
    raise(SIGSEGV);
    return;
  }
  std::fprintf(stderr, "smpc drop-in: device error word 0x%x after %s (info %u %u %u)\n", word,
               what, info[0], info[1], info[2]);
  std::fflush(stderr);
  std::abort();
}

smpc_ctx* ensure(Box& box) {
  BoxContext& bc = find(box);
  const unsigned n_mono = count_monomers(box);
  if (bc.ctx) {
    if (n_mono != bc.n_mono) {
      std::fprintf(stderr,
                   "smpc drop-in: the box's monomer count changed from %u to %u after the GPU "
                   "context was created\n",
                   bc.n_mono, n_mono);
      std::abort();
    }
    return bc.ctx;
  }
  smpc_replica_desc d{};
  for (int k = 0; k < 3; ++k) d.L[k] = box.BoxSize[k];
  d.n_fluid = bc.has_solvent ? static_cast<int>(bc.n_fluid) : 0;
  d.n_mono = static_cast<int>(n_mono);
  d.mol0_size = box.Molecules.empty() ? 0 : static_cast<int>(box.Molecules[0].Monomers.size());
  d.kT = bc.has_solvent ? bc.kT : (bc.md_kT > 0 ? bc.md_kT : box.Temperature);
  d.shear = bc.shear;
  d.h = 0.1;  // replaced by the dt of every MPC::step
  d.md_dt = bc.md_dt;
  d.lambda = box.Lambda;
  d.r_cut = box.Cutoff;
  d.r_verlet = box.VerletRadius;
  d.solvent_mass = 1.0;  // MPC.cpp:30
  d.seed = 1;
  d.potential = SMPC_POT_REF4824;

  smpc_options o{};
  o.precision = SMPC_FP64;
  o.rng = SMPC_RNG_INJECT;  // draws come from the reference's Rand stream
  o.mono_bin = SMPC_MONOBIN_REFERENCE;
  o.delrx_mode = SMPC_DELRX_REFERENCE;
  o.step_update = static_cast<int>(bc.step_update);
  o.max_neighbors = 0;
  o.strict_cells = 1;
  o.device = device_ordinal();
  o.angular_momentum = bc.angular_momentum ? 1 : 0;
  o.md_thermostat = bc.md_thermostat;
  o.andersen_nu = bc.andersen_nu;
  o.lowe_radius = bc.lowe_radius;
  smpc_ctx* ctx = nullptr;
  int rc = smpc_create(&d, 1, &o, &ctx);
  if (rc != SMPC_OK) fail(ctx, "smpc_create", rc);
  bc.ctx = ctx;
  bc.n_mono = n_mono;

  if (n_mono) {
    std::vector<double> pos, vel, force, mass;
    std::vector<int> amphi, anchor;
    flatten(box, pos, vel, &force);
    std::unordered_map<const MDParticle*, int> index;
    int k = 0;
    for (const auto& mol : box.Molecules)
      for (const auto& mono : mol.Monomers) {
        index[&mono] = k++;
        mass.push_back(mono.Mass);
        amphi.push_back(mono.AmphiType ? 1 : 0);
        anchor.push_back(mono.Anchor ? 1 : 0);
      }
    check(ctx, "smpc_set_monomers",
          smpc_set_monomers(ctx, 0, pos.data(), vel.data(), force.data(), mass.data(),
                            amphi.data(), anchor.data()));
    // directed bonds in MDParticle::Neighbors order (Molecule.cpp:146-157)
    std::vector<int> src, dst;
    for (const auto& mol : box.Molecules)
      for (const auto& mono : mol.Monomers)
        for (const MDParticle* nb : mono.Neighbors) {
          src.push_back(index.at(&mono));
          dst.push_back(index.at(nb));
        }
    check(ctx, "smpc_set_bonds",
          smpc_set_bonds(ctx, 0, static_cast<int>(src.size()), src.data(), dst.data()));
  }
  return ctx;
}

void upload_monomer_state(Box& box) {
  BoxContext& bc = find(box);
  if (!bc.n_mono) return;
  std::vector<double> pos, vel;
  flatten(box, pos, vel, nullptr);
  check(bc.ctx, "smpc_set_monomer_state_all",
        smpc_set_monomer_state_all(bc.ctx, pos.data(), vel.data()));
}

void download_monomer_state(Box& box, bool with_force) {
  BoxContext& bc = find(box);
  if (!bc.n_mono) return;
  std::vector<double> pos(3 * static_cast<size_t>(bc.n_mono)), vel(pos.size()),
      force(with_force ? pos.size() : 0);
  check(bc.ctx, "smpc_get_monomer_state_all",
        smpc_get_monomer_state_all(bc.ctx, pos.data(), vel.data(),
                                   with_force ? force.data() : nullptr));
  size_t k = 0;
  for (auto& mol : box.Molecules)
    for (auto& mono : mol.Monomers) {
      for (int d = 0; d < 3; ++d) {
        mono.Position(d) = pos[3 * k + d];
        mono.Velocity(d) = vel[3 * k + d];
        if (with_force) mono.Force(d) = force[3 * k + d];
      }
      ++k;
    }
}

void md_step(Box& box, bool calc_epot) {
  BoxContext& bc = find(box);
  smpc_ctx* ctx = ensure(box);
  if (!bc.md_ready) {
    if (!bc.mono_on_device) upload_monomer_state(box);
    check(ctx, "smpc_init_md", smpc_init_md(ctx));
    bc.md_ready = true;
    bc.mono_on_device = true;
  }
  check(ctx, "smpc_md_substeps", smpc_md_substeps(ctx, 1, calc_epot ? 1 : 0));
  if (!calc_epot) return;
  check_device(ctx, "md_step");
  download_monomer_state(box, true);
  double epot = 0.;
  check(ctx, "smpc_epot", smpc_epot(ctx, 0, &epot));
  // the device sums the potential energy over all molecules; Box::print_Epot
  // (Box.cpp:605-613) reads the sum over Molecules
  for (auto& mol : box.Molecules) mol.Epot = 0.0;
  if (!box.Molecules.empty()) box.Molecules[0].Epot = epot;
}

}  // namespace smpc_dropin
