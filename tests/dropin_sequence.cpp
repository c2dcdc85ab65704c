// The drop-in MPC's call sequence through the C ABI, as a C++ program that
// sees include/smpc.h and libsmpc.so only.
//
// starpolymersmd_gb300/dropin/ replaces the reference's MPC and thermostat
// classes (MPC.cpp, Thermostat_None.cpp) and needs the reference's own headers
// to compile, so it builds inside a reference checkout. This program makes the
// same calls in the same order with the same host logic, driven by a file that
// stands in for the reference's Box and Rand:
//   ensure()      smpc_create (the drop-in's options), smpc_set_fluid,
//                 smpc_set_monomers, smpc_set_bonds        (smpc_box.cpp)
//   md_step()     smpc_init_md once, smpc_md_substeps(1, calc_epot),
//                 error word, smpc_get_monomer_state_all, smpc_epot
//   MPC::step()   host delrx advance (MPC.cpp:117-118), on a collision step
//                 smpc_set_delrx, the grid shift drawn as the reference draws
//                 it (MPC.cpp:123), smpc_mpc_bin, smpc_cell_counts, per cell a
//                 gamma variate when the cell holds two or more particles then
//                 phi and theta (MPC.cpp:128-136, 244-245, 284-289), taken in
//                 that order from a recorded Rand tape, smpc_mpc_collide,
//                 error word                                (MPC_gpu.cpp)
//   MPC::pull()   smpc_get_fluid, smpc_cell_members, and the MPCCellList /
//                 MPCCellListFluidParticles rebuild the per-cell getters read
//                 (calculateEkinInCell, filledCells; MPC.cpp:335-418)
// A wrong occupancy would take the wrong number of draws off the tape and
// shift every later draw, so the occupancies are checked by the results.
//
// usage: dropin_sequence --shift-order            prints the order in which
//                                                 this build evaluates the
//                                                 three shift draws
//        dropin_sequence <input> <output>
// Input (native-endian): int32 L[3], n_fluid, n_mono, n_bond, n_loop,
// step_update, with_md, n_tape; float64 kT, shear, h, md_dt, lambda, r_cut,
// r_verlet; float64 fluid pos[3n], vel[3n]; monomer pos[3m], vel[3m],
// force[3m], mass[m]; int32 amphi[m], anchor[m], bond src[b], dst[b];
// float64 tape[n_tape] (Rand::real_uniform / real_gamma values in draw order).
// Output: float64 records, per loop step t: host delrx, device delrx, epot,
// monomer pos[3m], vel[3m], force[3m]; after a collision also: occupancies
// [cells], solvent pos[3n], vel[3n], fluid cell[n], monomer cell[m], device
// temperature, mirror kinetic energy (calculateEkinTotal), mirror filled
// cells; at the end the number of tape entries taken.
#include <csignal>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string_view>
#include <vector>

#include "smpc.h"

namespace {

struct Input {
  int L[3], n_fluid, n_mono, n_bond, n_loop, step_update, with_md, n_tape;
  double kT, shear, h, md_dt, lambda, r_cut, r_verlet;
  std::vector<double> fpos, fvel, mpos, mvel, mforce, mass, tape;
  std::vector<int> amphi, anchor, src, dst;
};

template <class T>
void read_into(std::FILE* f, T* p, size_t n) {
  if (n && std::fread(p, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "dropin_sequence: short input\n");
    std::exit(2);
  }
}

// stands in for the reference's Rand: values recorded from its stream
struct Tape {
  const std::vector<double>* v = nullptr;
  size_t pos = 0;
  double next() {
    if (pos >= v->size()) {
      std::fprintf(stderr, "dropin_sequence: Rand tape exhausted at %zu\n", pos);
      std::exit(3);
    }
    return (*v)[pos++];
  }
} g_rand;

double real_uniform() { return g_rand.next(); }
double real_gamma(double, double) { return g_rand.next(); }

// the shift's three components, built by the same expression shape as
// MPC.cpp:123 (a constructor taking three draws)
struct Vec3 {
  double x[3];
  Vec3(double a, double b, double c) : x{a, b, c} {}
};

int g_counter = 0;
double counted() { return static_cast<double>(g_counter++); }

[[noreturn]] void fail(smpc_ctx* ctx, const char* what, int rc) {
  std::fprintf(stderr, "smpc drop-in: %s failed (code %d): %s\n", what, rc,
               ctx ? smpc_last_error(ctx) : "no context");
  std::exit(4);
}

void check_device(smpc_ctx* ctx, const char* what) {
  unsigned word = 0, info[3] = {0, 0, 0};
  const int rc = smpc_error_word(ctx, &word, info);
  if (rc != SMPC_OK) fail(ctx, "smpc_error_word", rc);
  if (!word) return;
  if (word & (SMPC_ERR_FLUID_CELL | SMPC_ERR_MONO_CELL)) {
    // the reference prints the offender and raises SIGSEGV
    std::printf("CellIndex of %s out of range! (device error word %u, particle %u, %s)\n",
                (word & SMPC_ERR_FLUID_CELL) ? "fluid" : "monomer", word, info[0], what);
    std::fflush(stdout);
    std::raise(SIGSEGV);
  }
  std::fprintf(stderr, "smpc drop-in: device error word 0x%x after %s (info %u %u %u)\n", word,
               what, info[0], info[1], info[2]);
  std::exit(5);
}

void check(smpc_ctx* ctx, const char* what, int rc) {
  if (rc == SMPC_E_DEVICE) check_device(ctx, what);
  if (rc != SMPC_OK) fail(ctx, what, rc);
}

struct Driver {
  const Input& in;
  smpc_ctx* ctx = nullptr;
  bool md_ready = false;
  double delrx = 0.0;
  unsigned n_cells;
  std::vector<unsigned> cell_total;
  std::vector<double> draw_gamma, draw_phi, draw_theta;
  // host mirror (MPC.h:40-41): solvent and monomer state and the cell lists
  std::vector<double> fpos, fvel, mpos, mvel, mforce;
  std::vector<std::vector<int>> cell_list;  // >= 0 solvent id, < 0 monomer -(id + 1)
  std::vector<unsigned> cell_fluid;
  double epot = 0.0;

  explicit Driver(const Input& i)
      : in(i),
        n_cells(static_cast<unsigned>(i.L[0] * i.L[1] * i.L[2])),
        cell_total(n_cells),
        draw_gamma(n_cells),
        draw_phi(n_cells),
        draw_theta(n_cells),
        fpos(i.fpos),
        fvel(i.fvel),
        mpos(i.mpos),
        mvel(i.mvel),
        mforce(i.mforce),
        cell_list(n_cells),
        cell_fluid(n_cells) {}

  // smpc_box.cpp ensure()
  void ensure() {
    if (ctx) return;
    smpc_replica_desc d{};
    for (int k = 0; k < 3; ++k) d.L[k] = in.L[k];
    d.n_fluid = in.n_fluid;
    d.n_mono = in.n_mono;
    d.mol0_size = in.n_mono;
    d.kT = in.kT;
    d.shear = in.shear;
    d.h = 0.1;
    d.md_dt = in.md_dt;
    d.lambda = in.lambda;
    d.r_cut = in.r_cut;
    d.r_verlet = in.r_verlet;
    d.solvent_mass = 1.0;
    d.seed = 1;
    d.potential = SMPC_POT_REF4824;
    smpc_options o{};
    o.precision = SMPC_FP64;
    o.rng = SMPC_RNG_INJECT;
    o.mono_bin = SMPC_MONOBIN_REFERENCE;
    o.delrx_mode = SMPC_DELRX_REFERENCE;
    o.step_update = in.step_update;
    o.max_neighbors = 0;
    o.strict_cells = 1;
    o.device = 0;
    o.md_thermostat = SMPC_MDTHERMO_NONE;
    const int rc = smpc_create(&d, 1, &o, &ctx);
    if (rc != SMPC_OK) fail(ctx, "smpc_create", rc);
    if (smpc_n_cells(ctx, 0) != static_cast<int>(n_cells)) fail(ctx, "smpc_n_cells", -1);
    check(ctx, "smpc_set_fluid", smpc_set_fluid(ctx, 0, fpos.data(), fvel.data()));
    if (in.n_mono) {
      check(ctx, "smpc_set_monomers",
            smpc_set_monomers(ctx, 0, mpos.data(), mvel.data(), mforce.data(), in.mass.data(),
                              in.amphi.data(), in.anchor.data()));
      check(ctx, "smpc_set_bonds",
            smpc_set_bonds(ctx, 0, in.n_bond, in.src.data(), in.dst.data()));
    }
  }

  void download_monomer_state(bool with_force) {
    if (!in.n_mono) return;
    check(ctx, "smpc_get_monomer_state_all",
          smpc_get_monomer_state_all(ctx, mpos.data(), mvel.data(),
                                     with_force ? mforce.data() : nullptr));
  }

  // smpc_box.cpp md_step(): one Thermostat propagate
  void md_step(bool calc_epot) {
    ensure();
    if (!md_ready) {
      check(ctx, "smpc_init_md", smpc_init_md(ctx));
      md_ready = true;
    }
    check(ctx, "smpc_md_substeps", smpc_md_substeps(ctx, 1, calc_epot ? 1 : 0));
    if (!calc_epot) return;
    check_device(ctx, "md_step");
    download_monomer_state(true);
    check(ctx, "smpc_epot", smpc_epot(ctx, 0, &epot));
  }

  // MPC_gpu.cpp MPC::step(); returns whether it collided
  bool mpc_step(long t, double dt) {
    const double delrx_before = delrx;
    delrx += in.shear * in.L[1] * dt;
    delrx -= in.L[0] * std::round(delrx / in.L[0]);
    if (t % in.step_update) return false;
    ensure();
    check(ctx, "smpc_set_delrx", smpc_set_delrx(ctx, 0, delrx_before));
    Vec3 s(real_uniform() - 0.5, real_uniform() - 0.5, real_uniform() - 0.5);
    const double shift[3] = {s.x[0], s.x[1], s.x[2]};
    int collide_now = 0;
    check(ctx, "smpc_mpc_bin", smpc_mpc_bin(ctx, t, dt, shift, &collide_now));
    check_device(ctx, "MPC::sort");
    if (!collide_now) {
      std::fprintf(stderr, "MPC::step: device and host disagree on the collision step\n");
      std::exit(6);
    }
    check(ctx, "smpc_cell_counts", smpc_cell_counts(ctx, 0, cell_total.data(), nullptr));
    for (unsigned c = 0; c < n_cells; ++c) {
      const unsigned count = cell_total[c];
      draw_gamma[c] = count < 2 ? 0.0 : real_gamma(1.5 * (count - 1), in.kT);
      draw_phi[c] = real_uniform();
      draw_theta[c] = real_uniform();
    }
    smpc_inject inj{shift, draw_gamma.data(), draw_phi.data(), draw_theta.data()};
    check(ctx, "smpc_mpc_collide", smpc_mpc_collide(ctx, &inj));
    check_device(ctx, "MPC::collide");
    return true;
  }

  // MPC_gpu.cpp MPC::pull()
  void pull() {
    check(ctx, "smpc_get_fluid", smpc_get_fluid(ctx, 0, fpos.data(), fvel.data()));
    download_monomer_state(false);
    for (auto& l : cell_list) l.clear();
    for (auto& k : cell_fluid) k = 0;
    std::vector<int> fcell(in.n_fluid), mcell(in.n_mono);
    check(ctx, "smpc_cell_members",
          smpc_cell_members(ctx, 0, fcell.data(), in.n_mono ? mcell.data() : nullptr));
    for (int i = 0; i < in.n_fluid; ++i) {
      cell_list[fcell[i]].push_back(i);
      cell_fluid[fcell[i]]++;
    }
    for (int k = 0; k < in.n_mono; ++k)
      if (mcell[k] >= 0) cell_list[mcell[k]].push_back(-(k + 1));
    last_fcell.swap(fcell);
    last_mcell.swap(mcell);
  }
  std::vector<int> last_fcell, last_mcell;

  // MPC::calculateEkinInCell over the mirror (CMV with the monomers' masses)
  double ekin_in_cell(unsigned c) const {
    double cmv[3] = {0, 0, 0}, m = 0;
    for (int id : cell_list[c]) {
      const double* v = id >= 0 ? &fvel[3 * id] : &mvel[3 * (-id - 1)];
      const double w = id >= 0 ? 1.0 : in.mass[-id - 1];
      for (int d = 0; d < 3; ++d) cmv[d] += v[d] * w;
      m += w;
    }
    if (m > 0)
      for (double& x : cmv) x /= m;
    double e = 0;
    for (unsigned i = 0; i < cell_fluid[c]; ++i) {
      const double* v = &fvel[3 * cell_list[c][i]];
      double sq = 0;
      for (int d = 0; d < 3; ++d) sq += (v[d] - cmv[d]) * (v[d] - cmv[d]);
      e += sq;
    }
    return 0.5 * e;
  }
};

}  // namespace

int main(int argc, char** argv) {
  if (argc == 2 && std::string_view(argv[1]) == "--shift-order") {
    Vec3 s(counted(), counted(), counted());
    std::printf("%d %d %d\n", static_cast<int>(s.x[0]), static_cast<int>(s.x[1]),
                static_cast<int>(s.x[2]));
    return 0;
  }
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s --shift-order | <input> <output>\n", argv[0]);
    return 2;
  }
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  Input in;
  int hdr[11];
  read_into(f, hdr, 11);
  for (int k = 0; k < 3; ++k) in.L[k] = hdr[k];
  in.n_fluid = hdr[3];
  in.n_mono = hdr[4];
  in.n_bond = hdr[5];
  in.n_loop = hdr[6];
  in.step_update = hdr[7];
  in.with_md = hdr[8];
  in.n_tape = hdr[9];
  if (hdr[10] != 0x5350) {
    std::fprintf(stderr, "dropin_sequence: bad input tag\n");
    return 2;
  }
  double par[7];
  read_into(f, par, 7);
  in.kT = par[0];
  in.shear = par[1];
  in.h = par[2];
  in.md_dt = par[3];
  in.lambda = par[4];
  in.r_cut = par[5];
  in.r_verlet = par[6];
  const size_t n = in.n_fluid, m = in.n_mono, b = in.n_bond;
  in.fpos.resize(3 * n);
  in.fvel.resize(3 * n);
  in.mpos.resize(3 * m);
  in.mvel.resize(3 * m);
  in.mforce.resize(3 * m);
  in.mass.resize(m);
  in.amphi.resize(m);
  in.anchor.resize(m);
  in.src.resize(b);
  in.dst.resize(b);
  in.tape.resize(in.n_tape);
  read_into(f, in.fpos.data(), 3 * n);
  read_into(f, in.fvel.data(), 3 * n);
  read_into(f, in.mpos.data(), 3 * m);
  read_into(f, in.mvel.data(), 3 * m);
  read_into(f, in.mforce.data(), 3 * m);
  read_into(f, in.mass.data(), m);
  read_into(f, in.amphi.data(), m);
  read_into(f, in.anchor.data(), m);
  read_into(f, in.src.data(), b);
  read_into(f, in.dst.data(), b);
  read_into(f, in.tape.data(), in.tape.size());
  std::fclose(f);
  g_rand.v = &in.tape;

  Driver drv(in);
  std::vector<double> out;
  auto put = [&out](const double* p, size_t k) { out.insert(out.end(), p, p + k); };
  drv.ensure();
  for (long t = 0; t < in.n_loop; ++t) {
    if (in.with_md && m) drv.md_step(true);
    const bool collided = drv.mpc_step(t, in.h);
    double dev_delrx = 0;
    check(drv.ctx, "smpc_delrx", smpc_delrx(drv.ctx, 0, &dev_delrx));
    drv.download_monomer_state(true);
    out.push_back(drv.delrx);
    out.push_back(dev_delrx);
    out.push_back(drv.epot);
    put(drv.mpos.data(), 3 * m);
    put(drv.mvel.data(), 3 * m);
    put(drv.mforce.data(), 3 * m);
    if (!collided) continue;
    drv.pull();
    for (unsigned c = 0; c < drv.n_cells; ++c) out.push_back(drv.cell_total[c]);
    put(drv.fpos.data(), 3 * n);
    put(drv.fvel.data(), 3 * n);
    for (int c : drv.last_fcell) out.push_back(c);
    for (int c : drv.last_mcell) out.push_back(c);
    double T = 0;
    check(drv.ctx, "smpc_temperature", smpc_temperature(drv.ctx, 0, &T));
    out.push_back(T);
    double ekin = 0;
    unsigned filled = 0;
    for (unsigned c = 0; c < drv.n_cells; ++c) {
      ekin += drv.ekin_in_cell(c);
      filled += drv.cell_fluid[c] > 0;
    }
    out.push_back(ekin);
    out.push_back(filled);
  }
  check_device(drv.ctx, "end of run");
  out.push_back(static_cast<double>(g_rand.pos));
  smpc_destroy(drv.ctx);
  std::FILE* o = std::fopen(argv[2], "wb");
  if (!o || std::fwrite(out.data(), sizeof(double), out.size(), o) != out.size()) return 7;
  std::fclose(o);
  return 0;
}
