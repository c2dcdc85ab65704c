// C-callable harness around the StarPolymersMD reference classes, compiled
// together with the reference's own unmodified sources (see Makefile) into
// oracle/_ref/libsmpc_ref.so. Test infrastructure only: it lets Python build a
// system at library level the way star-polymers/src/mpc_test.cpp:73-110 and
// star-polymers/src/star-polymers.cpp:352-404 do, run the driver loop body
// (star-polymers.cpp:466,530,534: propagate, then MPC::step), and read or
// overwrite the state, the cell occupancies and the recorded random draws.
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>

#include "Box.h"
#include "MPC.h"
#include "Andersen_stochastic.h"
#include "Fourier_Autocorr.h"
#include "Lowe_Andersen.h"
#include "Thermostat_None.h"
#include "Vel_Autocorr_Fluid.h"
#include "Velocity_x.h"
#include "rand_tape.h"

namespace {

// Exposes the protected cell-list state of MPC (MPC.h:28-41) for read-out.
class HarnessMPC : public MPC {
 public:
  using MPC::MPC;
  unsigned cells() const { return NumberOfCells + 1; }
  unsigned cell_total(unsigned i) const { return static_cast<unsigned>(MPCCellList[i].size()); }
  unsigned cell_fluid(unsigned i) const { return MPCCellListFluidParticles[i]; }
  double get_delrx() const { return delrx; }
  void set_delrx(double d) { delrx = d; }
};

// The reference's solvent analyses (Analysis/Fourier_Autocorr.h,
// Analysis/Vel_Autocorr_Fluid.h) with their protected sums read out.
class HarnessFourier : public Fourier_Autocorr {
 public:
  using Fourier_Autocorr::Fourier_Autocorr;
  // modes18: the last sample's three modes (x, y, z components, re/im
  // interleaved); acf[3 * Entries]: Autocorrelation; counter: calculations
  void dump(double* modes18, double* acf, unsigned* counter) const {
    for (int j = 0; j < 3; ++j)
      for (int d = 0; d < 3; ++d) {
        modes18[6 * j + 2 * d] = Velocity_Fourier[j](d).real();
        modes18[6 * j + 2 * d + 1] = Velocity_Fourier[j](d).imag();
      }
    for (int i = 0; i < 3; ++i)
      for (unsigned e = 0; e < Entries; ++e)
        acf[i * Entries + e] = static_cast<double>(Autocorrelation[i][e]);
    *counter = Counter;
  }
};

class HarnessVacf : public Vel_Autocorr_Fluid {
 public:
  using Vel_Autocorr_Fluid::Vel_Autocorr_Fluid;
  // lag_sums[Entries]: Autocorrelation summed over particles (long double sums)
  void dump(double* lag_sums, unsigned* counter) const {
    for (unsigned e = 0; e < Entries; ++e) {
      long double s = 0.0L;
      for (unsigned i = 0; i < NumberOfParticles; ++i) s += Autocorrelation[i][e];
      lag_sums[e] = static_cast<double>(s);
    }
    *counter = Counter;
  }
};

struct RefSys {
  Box* box = nullptr;
  HarnessMPC* mpc = nullptr;
  Thermostat_None* thermo = nullptr;
  AndersenStochastic* andersen = nullptr;
  Lowe_Andersen* lowe = nullptr;
  Thermostat* active = nullptr;  // the one propagate() drives
  HarnessFourier* fourier = nullptr;
  HarnessVacf* vacf = nullptr;
};

int g_probe_counter = 0;
double probe_next() { return static_cast<double>(g_probe_counter++); }

}  // namespace

extern "C" {

RefSys* ref_create(int Lx, int Ly, int Lz, double T, double lambda, int Nc, double shear,
                   unsigned step_update, int amc) {
  RefSys* s = new RefSys();
  s->box = new Box(Lx, Ly, Lz, T, lambda);
  s->mpc = new HarnessMPC(*s->box, T, Nc, shear, step_update, amc != 0);
  return s;
}

void ref_destroy(RefSys* s) {
  delete s->lowe;
  delete s->fourier;
  delete s->vacf;
  delete s->thermo;
  delete s->andersen;
  delete s->mpc;
  delete s->box;
  delete s;
}

void ref_box_size(RefSys* s, int* L) {
  for (int i = 0; i < 3; ++i) L[i] = s->box->BoxSize[i];
}

void ref_add_star(RefSys* s, unsigned A, unsigned B, unsigned arms, double mass) {
  s->box->add_star(A, B, arms, mass);
}

void ref_make_thermostat(RefSys* s, double dt) {
  delete s->thermo;
  s->thermo = new Thermostat_None{*s->box, dt};
  s->active = s->thermo;
}

// The MPC-off integrator of star-polymers.cpp:387 (AndersenStochastic{box,
// StepSize, Temperature, 0.1}) with its temperature and frequency free.
void ref_make_andersen(RefSys* s, double dt, double T, double nu) {
  delete s->andersen;
  s->andersen = new AndersenStochastic{*s->box, dt, T, nu};
  s->active = s->andersen;
}

// Lowe_Andersen{box, dt, T, nu, r} (the MPC-off integrator star-polymers.cpp:388
// and gaussian_chain.cpp:382 construct with nu = 20, r = 1.5) as the
// propagating thermostat.
void ref_make_lowe_andersen(RefSys* s, double dt, double T, double nu, double r) {
  delete s->lowe;
  s->lowe = new Lowe_Andersen{*s->box, dt, T, nu, r};
  s->active = s->lowe;
}

void ref_mpc_initialize(RefSys* s) { s->mpc->initialize(); }

long ref_n_fluid(RefSys* s) { return static_cast<long>(s->mpc->Fluid.size()); }

int ref_n_mono(RefSys* s) {
  int n = 0;
  for (auto& mol : s->box->Molecules) n += static_cast<int>(mol.Monomers.size());
  return n;
}

void ref_get_fluid(RefSys* s, double* pos, double* vel) {
  long i = 0;
  for (auto& p : s->mpc->Fluid) {
    for (int d = 0; d < 3; ++d) {
      pos[3 * i + d] = p.Position(d);
      vel[3 * i + d] = p.Velocity(d);
    }
    ++i;
  }
}

void ref_set_fluid(RefSys* s, const double* pos, const double* vel) {
  long i = 0;
  for (auto& p : s->mpc->Fluid) {
    for (int d = 0; d < 3; ++d) {
      p.Position(d) = pos[3 * i + d];
      p.Velocity(d) = vel[3 * i + d];
    }
    ++i;
  }
}

void ref_get_monomers(RefSys* s, double* pos, double* vel, double* force, double* mass,
                      int* amphi, int* anchor) {
  int i = 0;
  for (auto& mol : s->box->Molecules) {
    for (auto& m : mol.Monomers) {
      for (int d = 0; d < 3; ++d) {
        if (pos) pos[3 * i + d] = m.Position(d);
        if (vel) vel[3 * i + d] = m.Velocity(d);
        if (force) force[3 * i + d] = m.Force(d);
      }
      if (mass) mass[i] = m.Mass;
      if (amphi) amphi[i] = m.AmphiType ? 1 : 0;
      if (anchor) anchor[i] = m.Anchor ? 1 : 0;
      ++i;
    }
  }
}

// Overwrites monomer positions and velocities, then rebuilds the Verlet lists
// and forces exactly as the Thermostat_None constructor does
// (Thermostat_None.cpp:5-12).
void ref_set_monomers(RefSys* s, const double* pos, const double* vel) {
  int i = 0;
  for (auto& mol : s->box->Molecules) {
    for (auto& m : mol.Monomers) {
      for (int d = 0; d < 3; ++d) {
        m.Position(d) = pos[3 * i + d];
        m.Velocity(d) = vel[3 * i + d];
      }
      ++i;
    }
  }
  s->box->update_VerletLists();
  s->box->calculate_forces_verlet();
}

// Directed FENE bonds as stored in MDParticle::Neighbors (Particle.h:57),
// global monomer indices. Returns the number of bonds; src/dst may be null.
int ref_get_bonds(RefSys* s, int* src, int* dst) {
  std::vector<const MDParticle*> base;
  int off = 0;
  std::vector<int> mol_off;
  for (auto& mol : s->box->Molecules) {
    mol_off.push_back(off);
    off += static_cast<int>(mol.Monomers.size());
  }
  int nb = 0;
  int mi = 0;
  for (auto& mol : s->box->Molecules) {
    const MDParticle* first = mol.Monomers.data();
    for (unsigned k = 0; k < mol.Monomers.size(); ++k) {
      for (auto* nbp : mol.Monomers[k].Neighbors) {
        if (src) src[nb] = mol_off[mi] + static_cast<int>(k);
        if (dst) dst[nb] = mol_off[mi] + static_cast<int>(nbp - first);
        ++nb;
      }
    }
    ++mi;
  }
  return nb;
}

void ref_propagate(RefSys* s, int calc_epot) { s->active->propagate(calc_epot != 0); }

void ref_mpc_step(RefSys* s, long t, double dt) { s->mpc->step(t, dt); }

unsigned ref_n_cells(RefSys* s) { return s->mpc->cells(); }

void ref_cell_counts(RefSys* s, unsigned* total, unsigned* fluid) {
  const unsigned n = s->mpc->cells();
  for (unsigned i = 0; i < n; ++i) {
    if (total) total[i] = s->mpc->cell_total(i);
    if (fluid) fluid[i] = s->mpc->cell_fluid(i);
  }
}

// MPCParticle::CellIndex of every solvent particle and monomer as the last
// MPC::sort set it (MPC.cpp:209, 224).
void ref_cell_index(RefSys* s, int* fluid_cell, int* mono_cell) {
  if (fluid_cell)
    for (size_t i = 0; i < s->mpc->Fluid.size(); ++i)
      fluid_cell[i] = static_cast<int>(s->mpc->Fluid[i].CellIndex);
  if (mono_cell) {
    int k = 0;
    for (auto& mol : s->box->Molecules)
      for (auto& mono : mol.Monomers) mono_cell[k++] = static_cast<int>(mono.CellIndex);
  }
}

double ref_delrx(RefSys* s) { return s->mpc->get_delrx(); }
void ref_set_delrx(RefSys* s, double d) { s->mpc->set_delrx(d); }

double ref_temperature(RefSys* s) { return s->mpc->calculateCurrentTemperature(); }

double ref_epot(RefSys* s) {
  double e = 0.0;
  for (auto& mol : s->box->Molecules) e += mol.Epot;
  return e;
}

// Box::center_of_mass_reference_frame + calculate_gyration_tensor
// (Box.cpp:81-102, 330-353): out[0] = R_g, out[1..9] = G (column-major).
void ref_gyration(RefSys* s, double* out) {
  s->box->center_of_mass_reference_frame();
  auto g = s->box->calculate_gyration_tensor();
  out[0] = std::get<0>(g);
  const Matrix3d& m = std::get<1>(g);
  for (int i = 0; i < 9; ++i) out[1 + i] = m.data()[i];
}

// Output-step observables of the star-polymers.cpp loop (:467-473) after
// Box::center_of_mass_reference_frame: out[0] = R_g, out[1..9] = G
// (row-major), out[10..12] = rotation frequency (Box.cpp:330-379),
// out[13] = kinetic energy (Box::calculate_ekin, Box.cpp:288-294), out[14] =
// the temperature Box::print_Ekin_and_Temperature prints (Box.cpp:635-646),
// out[15] = number of molecules.
void ref_observables(RefSys* s, double* out) {
  Box& b = *s->box;
  b.center_of_mass_reference_frame();
  auto g = b.calculate_gyration_tensor();
  out[0] = std::get<0>(g);
  const Matrix3d& m = std::get<1>(g);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out[1 + 3 * i + j] = m(i, j);
  const Vector3d w = b.calculate_rotation_frequency();
  for (int i = 0; i < 3; ++i) out[10 + i] = w(i);
  unsigned n = 0;
  for (auto& mol : b.Molecules) n += mol.NumberOfMonomers;
  out[13] = b.calculate_ekin();
  out[14] = out[13] * 2. / (3. * (n - 1));
  out[15] = static_cast<double>(b.Molecules.size());
}

// VelocityX (Velocity_x.h:76-100) applied to the solvent once, the way
// star-polymers.cpp:468,483 does (centre-of-mass frame first): per bin k of
// floor(p / width) along x and along y, (sum v_x, sum v_y, count) at
// out[3 * (k - k0)] with k0 = floor(-L / (2 width)) of the axis.
class HarnessVelocityX : public VelocityX {
 public:
  using VelocityX::VelocityX;
  void dump(double width, const std::map<double, vel_xy>& sums,
            const std::map<double, double>& counts, int L, double* out, int n) const {
    const long k0 = static_cast<long>(std::floor(-L / (2.0 * width)));
    for (int i = 0; i < 3 * n; ++i) out[i] = 0.0;
    for (const auto& kv : sums) {
      const long k = std::lround(kv.first / width) - k0;
      if (k < 0 || k >= n) continue;
      out[3 * k] = kv.second.vel_x;
      out[3 * k + 1] = kv.second.vel_y;
      out[3 * k + 2] = counts.at(kv.first);
    }
  }
  void dump_x(double w, int L, double* out, int n) const {
    dump(w, vel_x_average, vel_x_average_count, L, out, n);
  }
  void dump_y(double w, int L, double* out, int n) const {
    dump(w, vel_y_average, vel_y_average_count, L, out, n);
  }
};

void ref_velocity_profile(RefSys* s, double width, double* x_out, int n_x, double* y_out,
                          int n_y) {
  s->box->center_of_mass_reference_frame();
  HarnessVelocityX vx(*s->box, *s->mpc, width);
  (*s->mpc)(vx);
  vx.dump_x(width, s->box->BoxSize[0], x_out, n_x);
  vx.dump_y(width, s->box->BoxSize[1], y_out, n_y);
}

// Fourier_Autocorr / Vel_Autocorr_Fluid over every solvent particle, applied
// through MPC::operator() (MPC.h:110-115) once per sample.
void ref_fourier_start(RefSys* s, unsigned entries, double dt, double L) {
  delete s->fourier;
  s->fourier = new HarnessFourier(static_cast<unsigned>(s->mpc->Fluid.size()), entries, dt, L);
}
void ref_fourier_sample(RefSys* s) { (*s->mpc)(*s->fourier); }
void ref_fourier_dump(RefSys* s, double* modes18, double* acf, unsigned* counter) {
  s->fourier->dump(modes18, acf, counter);
}
void ref_vacf_start(RefSys* s, unsigned entries, double dt) {
  delete s->vacf;
  s->vacf = new HarnessVacf(static_cast<unsigned>(s->mpc->Fluid.size()), entries, dt);
}
void ref_vacf_sample(RefSys* s) { (*s->mpc)(*s->vacf); }
void ref_vacf_dump(RefSys* s, double* lag_sums, unsigned* counter) { s->vacf->dump(lag_sums, counter); }

// Runs the star-polymers.cpp loop body (lines 466/530 then 534) for
// t = t0 .. t0+n-1 without output; used to time the reference.
void ref_run(RefSys* s, long t0, long n, double mpc_dt, int with_md) {
  for (long t = t0; t < t0 + n; ++t) {
    if (with_md) s->active->propagate(false);
    s->mpc->step(t, mpc_dt);
  }
}

// The reference's restart files, written and read by its own code:
// MPC::print_fluid_complete (MPC.cpp:570-579), MPC::initialize(filename,
// Box_old) (MPC.cpp:57-113), Box::print_PDB_with_velocity (Box.cpp:563-602)
// and Molecule::star_from_file (Molecule.cpp:178-224) on molecule `mol`.
int ref_print_fluid_complete(RefSys* s, const char* path) {
  FILE* f = std::fopen(path, "w");
  if (!f) return 1;
  s->mpc->print_fluid_complete(f);
  std::fclose(f);
  return 0;
}

void ref_mpc_initialize_from_file(RefSys* s, const char* path, int Lx_old, int Ly_old,
                                  int Lz_old) {
  s->mpc->initialize(path, std::array<int, 3>{Lx_old, Ly_old, Lz_old});
}

int ref_print_pdb_with_velocity(RefSys* s, const char* path, int step) {
  FILE* f = std::fopen(path, "w");
  if (!f) return 1;
  s->box->print_PDB_with_velocity(f, step);
  std::fclose(f);
  return 0;
}

void ref_star_from_file(RefSys* s, int mol, const char* path, unsigned A, unsigned B,
                        unsigned arms, int set_zero) {
  s->box->Molecules[mol].star_from_file(path, A, B, arms, set_zero != 0);
}

// Reports which draw of "Vector3d(f() - 0.5, f() - 0.5, f() - 0.5)" lands in
// each component under this compiler (argument evaluation order is
// unspecified in C++); MPC.cpp:123 builds the grid shift this way.
void ref_shift_arg_order(int* order3) {
  g_probe_counter = 0;
  Vector3d v(probe_next() - 0.5, probe_next() - 0.5, probe_next() - 0.5);
  for (int i = 0; i < 3; ++i) order3[i] = static_cast<int>(v(i) + 0.5);
}

}  // extern "C"
