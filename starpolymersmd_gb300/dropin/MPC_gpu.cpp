// GPU MPC solvent behind the reference's MPC class interface (MPC.h in this
// directory). Reference behaviour each method reproduces is cited as
// star-polymers/lib/Hydrodynamics/MPC.cpp:line.
#include "MPC.h"

#include <cstdio>
#include <cstdlib>

#include "Box.h"
#include "smpc.h"
#include "smpc_box.h"

using smpc_dropin::check;
using smpc_dropin::check_device;

namespace {

// Draws one solvent particle of a freshly filled box the way MPC::initialize
// does (MPC.cpp:37-42): per axis a position uniform in the box, then a
// velocity component uniform in [-1/2, 1/2).
void draw_uniform_particle(MPCParticle& part, const std::array<int, 3>& L) {
  for (unsigned d = 0; d < 3; ++d) {
    part.Position(d) = L[d] * (Rand::real_uniform() - 0.5);
    part.Velocity(d) = Rand::real_uniform() - 0.5;
  }
}

// Restart filling of a grown box (MPC.cpp:79-88): new particles go into the
// added slabs, split evenly between both ends, or anywhere on an axis that
// did not grow.
void draw_restart_particle(MPCParticle& part, const std::array<int, 3>& L,
                           const std::array<int, 3>& L_old) {
  for (unsigned d = 0; d < 3; ++d) {
    double u = Rand::real_uniform();
    const int grown = L[d] - L_old[d];
    if (grown > 0)
      u = u < 0.5 ? -L[d] * 0.5 + grown * u : L_old[d] * 0.5 + grown * (u - 0.5);
    else
      u = L[d] * (u - 0.5);
    part.Position(d) = u;
    part.Velocity(d) = Rand::real_uniform() - 0.5;
  }
}

}  // namespace

// MPC.cpp:10-32
MPC::MPC(Box& box, double aTemperature, int N_c, double aShear, unsigned step, bool angular_mom)
    : Hydrodynamics{box},
      Temperature{aTemperature},
      Shear{aShear},
      step_update{step},
      angular_momentum{angular_mom} {
  NumberOfCells = SimBox.BoxSize[0] * SimBox.BoxSize[1] * SimBox.BoxSize[2] - 1;
  NumberOfMPCParticles = N_c * (NumberOfCells + 1);
  for (int d = 0; d < 3; ++d) BoxSize[d] = SimBox.BoxSize[d];
  MPCCellList.assign(NumberOfCells + 1, std::vector<MPCParticle*>());
  MPCCellListFluidParticles.assign(NumberOfCells + 1, 0);
  c = cos(130.0 * M_PI / 180.0);
  s = sin(130.0 * M_PI / 180.0);
  delrx = 0.;
  shear_on = Shear != 0.;
  Fluid.reserve(NumberOfMPCParticles);
  for (unsigned i = 0; i < NumberOfMPCParticles; ++i) Fluid.push_back(MPCParticle(1.0));
  cell_total.assign(NumberOfCells + 1, 0);
  draw_gamma.assign(NumberOfCells + 1, 0.0);
  draw_phi.assign(NumberOfCells + 1, 0.0);
  draw_theta.assign(NumberOfCells + 1, 0.0);

  smpc_dropin::BoxContext& bc = smpc_dropin::attach(SimBox);
  bc.has_solvent = true;
  bc.kT = Temperature;
  bc.shear = Shear;
  bc.step_update = step_update;
  bc.n_fluid = NumberOfMPCParticles;
  bc.angular_momentum = angular_momentum;
}

MPC::~MPC() { smpc_dropin::detach(SimBox); }

void MPC::on_device(const char* what) const {
  std::fprintf(stderr,
               "MPC::%s: this phase runs on the GPU inside MPC::step and is not callable on "
               "its own\n",
               what);
  std::abort();
}

// MPC.cpp:34-55
void MPC::initialize() {
  Vector3d CMV(0., 0., 0.);
  for (auto& part : Fluid) {
    draw_uniform_particle(part, BoxSize);
    wrap(part);
    CMV += part.Velocity;
  }
  CMV /= NumberOfMPCParticles;
  for (auto& part : Fluid) part.Velocity -= CMV;
  fluid_dirty = true;
  host_stale = false;
}

// MPC.cpp:57-113: restart from an end_fluid file written by
// print_fluid_complete, refilling particles that are missing or lie outside
// the (possibly grown) box.
void MPC::initialize(string filename, std::array<int, 3> Box_old) {
  std::fstream file{filename};
  Vector3d pos{Vector3d::Zero()};
  Vector3d vel{Vector3d::Zero()};
  Vector3d CMV(0., 0., 0.);
  int from_file = 0, added = 0;
  for (auto& part : Fluid) {
    bool have = static_cast<bool>(file >> pos(0) >> pos(1) >> pos(2) >> vel(0) >> vel(1) >> vel(2));
    if (have) {
      bool outside = false;
      for (int d = 0; d < 3; ++d) outside = outside || fabs(round(pos(d) / BoxSize[d])) >= 1.0;
      have = !outside;
    }
    if (have) {
      part.Position = pos;
      part.Velocity = vel;
      ++from_file;
    } else {
      draw_restart_particle(part, BoxSize, Box_old);
      ++added;
    }
    wrap(part);
    CMV += part.Velocity;
  }
  std::cout << "# fluid particles from file: " << from_file << "# fluid particles added: " << added
            << std::endl;
  CMV /= NumberOfMPCParticles;
  for (auto& part : Fluid) part.Velocity -= CMV;
  fluid_dirty = true;
  host_stale = false;
}

// MPC.cpp:116-142. The delrx advance happens on every call, on the host; on a
// collision step the device runs recentring, streaming, the grid shift and
// the counting sort (smpc_mpc_bin), the host draws the per-cell random
// numbers from Rand in the reference's order using the occupancies, and the
// device runs the thermostat + rotation and the unshift (smpc_mpc_collide).
void MPC::step(const long int& t, const double& dt) {
  const double delrx_before = delrx;
  delrx += Shear * BoxSize[1] * dt;
  delrx -= BoxSize[0] * round(delrx / BoxSize[0]);
  if (t % step_update) return;
  smpc_dropin::BoxContext& bc = smpc_dropin::find(SimBox);
  smpc_ctx* ctx = smpc_dropin::ensure(SimBox);
  if (fluid_dirty) {
    std::vector<double> pos(3 * Fluid.size()), vel(3 * Fluid.size());
    for (size_t i = 0; i < Fluid.size(); ++i)
      for (int d = 0; d < 3; ++d) {
        pos[3 * i + d] = Fluid[i].Position(d);
        vel[3 * i + d] = Fluid[i].Velocity(d);
      }
    check(ctx, "smpc_set_fluid", smpc_set_fluid(ctx, 0, pos.data(), vel.data()));
    fluid_dirty = false;
  }
  if (!bc.mono_on_device) smpc_dropin::upload_monomer_state(SimBox);
  check(ctx, "smpc_set_delrx", smpc_set_delrx(ctx, 0, delrx_before));

  // MPC.cpp:123: the same expression, so that the compiler evaluates the three
  // draws in the same order as it does for the reference
  Vector3d Shift(Rand::real_uniform() - 0.5, Rand::real_uniform() - 0.5, Rand::real_uniform() - 0.5);
  const double shift[3] = {Shift(0), Shift(1), Shift(2)};
  int collide_now = 0;
  check(ctx, "smpc_mpc_bin", smpc_mpc_bin(ctx, t, dt, shift, &collide_now));
  check_device(ctx, "MPC::sort");
  if (!collide_now) {
    std::fprintf(stderr, "MPC::step: device and host disagree on the collision step\n");
    std::abort();
  }
  check(ctx, "smpc_cell_counts", smpc_cell_counts(ctx, 0, cell_total.data(), nullptr));
  // MPC.cpp:128-136 in cell order: thermostat (a gamma variate when the cell
  // holds two or more particles, MPC.cpp:284-289), then collide (phi, theta,
  // MPC.cpp:244-245) for every cell, empty ones included
  for (unsigned Index = 0; Index <= NumberOfCells; ++Index) {
    const unsigned count = cell_total[Index];
    draw_gamma[Index] = count < 2 ? 0.0 : Rand::real_gamma(1.5 * (count - 1), Temperature);
    draw_phi[Index] = Rand::real_uniform();
    draw_theta[Index] = Rand::real_uniform();
  }
  smpc_inject inj{shift, draw_gamma.data(), draw_phi.data(), draw_theta.data()};
  check(ctx, "smpc_mpc_collide", smpc_mpc_collide(ctx, &inj));
  check_device(ctx, "MPC::collide");
  if (!bc.mono_on_device) smpc_dropin::download_monomer_state(SimBox, false);
  host_stale = true;
  collided = true;
}

// Refreshes the host mirror: solvent state, CellIndex of every particle and
// the cell lists of the last sort, in the reference's list order (solvent in
// Fluid order, then monomers molecule by molecule, MPC.cpp:207-236).
void MPC::pull() const {
  if (!host_stale) return;
  smpc_dropin::BoxContext& bc = smpc_dropin::find(SimBox);
  smpc_ctx* ctx = bc.ctx;
  const size_t n = Fluid.size();
  std::vector<double> pos(3 * n), vel(3 * n);
  check(ctx, "smpc_get_fluid", smpc_get_fluid(ctx, 0, pos.data(), vel.data()));
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      Fluid[i].Position(d) = pos[3 * i + d];
      Fluid[i].Velocity(d) = vel[3 * i + d];
    }
  if (bc.mono_on_device) smpc_dropin::download_monomer_state(SimBox, false);
  for (auto& list : MPCCellList) list.clear();
  for (auto& k : MPCCellListFluidParticles) k = 0;
  if (collided) {
    std::vector<int> fcell(n), mcell(bc.n_mono);
    check(ctx, "smpc_cell_members",
          smpc_cell_members(ctx, 0, fcell.data(), bc.n_mono ? mcell.data() : nullptr));
    for (size_t i = 0; i < n; ++i) {
      Fluid[i].CellIndex = static_cast<unsigned>(fcell[i]);
      MPCCellList[fcell[i]].push_back(&Fluid[i]);
      MPCCellListFluidParticles[fcell[i]]++;
    }
    size_t k = 0;
    for (auto& mol : SimBox.Molecules)
      for (auto& mono : mol.Monomers) {
        const int cell = mcell[k++];
        if (cell < 0) continue;
        mono.CellIndex = static_cast<unsigned>(cell);
        MPCCellList[cell].push_back(&mono);
      }
  }
  host_stale = false;
}

void MPC::streaming(const double&) { on_device("streaming"); }
void MPC::sort() { on_device("sort"); }
void MPC::collide(unsigned, const Vector3d&) { on_device("collide"); }
void MPC::thermostat(unsigned, const Vector3d&) { on_device("thermostat"); }
void MPC::periodic_image_box(unsigned) { on_device("periodic_image_box"); }
void MPC::undo_periodic_image_box(unsigned) { on_device("undo_periodic_image_box"); }
void MPC::check_bounds() { on_device("check_bounds"); }
void MPC::shiftParticles(const Vector3d&) { on_device("shiftParticles"); }

// ---------------------------------------------------------------- per-cell getters
// MPC.cpp:314-418, over the host mirror of the last sort.

void MPC::calculateCMV(unsigned Index, Vector3d& CMV) {
  pull();
  CMV = Vector3d(0., 0., 0.);
  double mass = 0.;
  for (MPCParticle* p : MPCCellList[Index]) {
    CMV += p->Velocity * p->Mass;
    mass += p->Mass;
  }
  if (mass > 0) CMV /= mass;
}

void MPC::calculateCMP(unsigned Index, Vector3d& CMP) {
  pull();
  CMP = Vector3d(0., 0., 0.);
  double mass = 0.;
  for (MPCParticle* p : MPCCellList[Index]) {
    CMP += p->Position * p->Mass;
    mass += p->Mass;
  }
  if (mass > 0) CMP /= mass;
}

void MPC::calculateFluidVelocity(unsigned Index, Vector3d& FluidVelocity) {
  pull();
  FluidVelocity = Vector3d(0., 0., 0.);
  const unsigned nf = MPCCellListFluidParticles[Index];
  for (unsigned i = 0; i < nf; ++i) FluidVelocity += MPCCellList[Index][i]->Velocity;
  if (nf > 0) FluidVelocity /= static_cast<double>(nf);
}

// Angular-momentum correction of one cell (MPC.cpp:343-374): inertia tensor
// about the cell's centre of mass, solved against the angular momentum the
// rotation removed.
void MPC::calculateAngular(unsigned Index, Vector3d& Angular, const Vector3d& CMV,
                           const Vector3d& CMP, const Matrix3d& Rotation) {
  pull();
  Vector3d lost(0., 0., 0.);
  Matrix3d I = Matrix3d::Zero();
  for (MPCParticle* p : MPCCellList[Index]) {
    const Vector3d r = p->Position - CMP;
    const Vector3d u = p->Velocity - CMV;
    lost += p->Mass * r.cross(u - Rotation * u);
    I(0, 0) += p->Mass * (pow(r(1), 2) + pow(r(2), 2));
    I(1, 1) += p->Mass * (pow(r(0), 2) + pow(r(2), 2));
    I(2, 2) += p->Mass * (pow(r(1), 2) + pow(r(0), 2));
    I(0, 1) -= p->Mass * r(0) * r(1);
    I(0, 2) -= p->Mass * r(0) * r(2);
    I(1, 2) -= p->Mass * r(1) * r(2);
  }
  I(1, 0) = I(0, 1);
  I(2, 0) = I(0, 2);
  I(2, 1) = I(1, 2);
  Angular = I.llt().solve(lost);
}

void MPC::calculateAngularMomentum(unsigned Index, Vector3d& L, const Vector3d& CMV,
                                   const Vector3d& CMP) {
  pull();
  L = Vector3d(0., 0., 0.);
  for (MPCParticle* p : MPCCellList[Index])
    L += p->Mass * (p->Position - CMP).cross(p->Velocity - CMV);
}

double MPC::calculateEkinInCell(unsigned Index) {
  Vector3d CMV{};
  calculateCMV(Index, CMV);
  double ekin = 0.;
  const unsigned nf = MPCCellListFluidParticles[Index];
  for (unsigned i = 0; i < nf; ++i) {
    const MPCParticle* p = MPCCellList[Index][i];
    ekin += p->Mass * (p->Velocity - CMV).squaredNorm();
  }
  return 0.5 * ekin;
}

double MPC::calculateEkinTotal() {
  double ekin = 0.;
  for (unsigned i = 0; i <= NumberOfCells; ++i) ekin += calculateEkinInCell(i);
  return ekin;
}

// MPC.cpp:405-409 on the device: solvent kinetic energy about each cell's
// centre-of-mass velocity (monomers included in the CMV) over the solvent's
// degrees of freedom minus the filled cells.
double MPC::calculateCurrentTemperature() {
  if (!collided) return 0.0;  // no cell lists yet: the reference sums nothing
  smpc_dropin::BoxContext& bc = smpc_dropin::find(SimBox);
  if (!bc.mono_on_device) smpc_dropin::upload_monomer_state(SimBox);
  double T = 0.;
  check(bc.ctx, "smpc_temperature", smpc_temperature(bc.ctx, 0, &T));
  return T;
}

unsigned MPC::filledCells() {
  pull();
  unsigned n = 0;
  for (unsigned i = 0; i <= NumberOfCells; ++i) n += MPCCellListFluidParticles[i] > 0;
  return n;
}

// ---------------------------------------------------------------- boundary helpers
// Lees-Edwards and periodic wraps (MPC.cpp:421-530), pure functions of the
// host's delrx, which follows the device's step for step.

void MPC::LEBC(Particle& part) { LEBC(part.Position, part.Velocity); }

void MPC::LEBC(Vector3d& pos, Vector3d& vel) {
  const double cy = round(pos(1) / BoxSize[1]);
  pos(0) -= BoxSize[0] * round(pos(0) / BoxSize[0]);
  pos(0) -= cy * delrx;
  pos(0) -= BoxSize[0] * round(pos(0) / BoxSize[0]);
  pos(1) -= BoxSize[1] * cy;
  pos(2) -= BoxSize[2] * round(pos(2) / BoxSize[2]);
  vel(0) -= cy * Shear * BoxSize[1];
}

void MPC::LEBC_to_zero(Vector3d& pos, Vector3d& vel) { LEBC(pos, vel); }

Vector3d MPC::relative_position(Particle& one, Particle& two) {
  return relative_position(one.Position, two.Position);
}

Vector3d MPC::relative_position(const Vector3d one, const Vector3d two) {
  Vector3d r{two - one};
  const double cy = round(r(1) / BoxSize[1]);
  r(0) -= BoxSize[0] * round(r(0) / BoxSize[0]);
  r(0) -= cy * delrx;
  r(0) -= BoxSize[0] * round(r(0) / BoxSize[0]);
  r(1) -= BoxSize[1] * cy;
  r(2) -= BoxSize[2] * round(r(2) / BoxSize[2]);
  return r;
}

Vector3d& MPC::wrap(Vector3d& pos) {
  for (unsigned d = 0; d < 3; ++d) pos(d) -= round(pos(d) / BoxSize[d]) * BoxSize[d];
  return pos;
}

Vector3d MPC::wrap(Vector3d&& pos) {
  for (unsigned d = 0; d < 3; ++d) pos(d) -= round(pos(d) / BoxSize[d]) * BoxSize[d];
  return pos;
}

void MPC::wrap(Particle& part) {
  if (shear_on)
    LEBC(part);
  else
    wrap(part.Position);
}

void MPC::wrap(Vector3d& pos, Vector3d& vel) {
  if (shear_on)
    LEBC(pos, vel);
  else
    wrap(pos);
}

Vector3d& MPC::wrap_to_zero(Vector3d& pos) { return wrap(pos); }

void MPC::wrap_to_zero(Particle& part) { wrap(part.Position, part.Velocity); }

void MPC::wrap_to_zero(Vector3d& pos, Vector3d& vel) { wrap(pos, vel); }

// ---------------------------------------------------------------- output
// Text formats of MPC.cpp:533-579, so existing post-processing reads them.

void MPC::print_fluid(FILE* f, int step, int z_start, int z_stop) {
  std::fprintf(f, "TIME %d \n", step);
  for (int z = z_start; z <= z_stop; ++z) {
    std::fprintf(f, "Z %d \n", z);
    for (int x = 0; x < BoxSize[0]; ++x) std::fprintf(f, "%f ", x + 0.5);
    std::fprintf(f, "\n");
    for (int y = 0; y < BoxSize[1]; ++y) std::fprintf(f, "%f ", y + 0.5);
    std::fprintf(f, "\n");
    for (int x = 0; x < BoxSize[0]; ++x) {
      for (int y = 0; y < BoxSize[1]; ++y) {
        Vector3d v{};
        calculateFluidVelocity(x + BoxSize[0] * y + BoxSize[0] * BoxSize[1] * z, v);
        std::fprintf(f, "%f %f ", v(0), v(1));
      }
      std::fprintf(f, "\n");
    }
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "\n");
}

void MPC::print_fluid_with_coordinates(FILE* f, int step, int z_start, int z_stop) {
  std::fprintf(f, "TIME     %d \n", step);
  for (int z = z_start; z < z_stop; ++z)
    for (int x = 0; x < BoxSize[0]; ++x)
      for (int y = 0; y < BoxSize[1]; ++y) {
        Vector3d v{};
        calculateFluidVelocity(x + BoxSize[0] * y + BoxSize[0] * BoxSize[1] * z, v);
        std::fprintf(f, "%f %f %f %f %f %f \n", x + 0.5, y + 0.5, z + 0.5, v(0), v(1), v(2));
      }
  std::fprintf(f, "\n");
}

void MPC::print_fluid_complete(FILE* f) {
  pull();
  for (const auto& part : Fluid)
    std::fprintf(f, "%f %f %f %f %f %f \n", part.Position(0), part.Position(1), part.Position(2),
                 part.Velocity(0), part.Velocity(1), part.Velocity(2));
}
