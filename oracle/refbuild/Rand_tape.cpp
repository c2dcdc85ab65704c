// Project-written implementation of the reference's unchanged Rand.h
// (star-polymers/lib/Rand.h:10-29), used only to build the CPU oracle.
// The engine and distributions are the same libstdc++ objects with the same
// seed as star-polymers/lib/Rand.cpp:6-11 (mt19937_64 seeded with 1,
// default-constructed distributions, gamma re-parameterised per call as at
// Rand.cpp:40-43), so the stream of values is the reference's own. Every value
// handed out is also appended to an in-memory tape (rand_tape.h) so that a
// collision's shift, axes and gamma variates can be injected elsewhere.
#include "Rand.h"

#include <vector>

#include "rand_tape.h"

mt19937_64 Rand::generator(1);
normal_distribution<double> Rand::dis_normal;
uniform_real_distribution<double> Rand::dis_uniform;
uniform_int_distribution<int> Rand::dis_intuniform;
chi_squared_distribution<double> Rand::dis_chisquared;
gamma_distribution<double> Rand::dis_gamma;

namespace {
struct TapeEntry {
  double value;
  int kind;
};
std::vector<TapeEntry> g_tape;
bool g_tape_on = false;

unsigned long long g_pending_seed = 1;

inline double logged(double v, int kind) {
  if (g_tape_on) g_tape.push_back(TapeEntry{v, kind});
  return v;
}
}  // namespace

// Rand::init() is declared by Rand.h but never defined or called by the
// reference; here it re-seeds the engine with the seed requested through
// rand_tape_reseed() and clears the distributions' cached state, which lets
// one process generate several independent fixtures.
void Rand::init() {
  generator.seed(g_pending_seed);
  dis_normal.reset();
  dis_uniform.reset();
  dis_intuniform.reset();
  dis_chisquared.reset();
  dis_gamma.reset();
}

double Rand::real_normal() { return logged(dis_normal(generator), TAPE_NORMAL); }

double Rand::real_normal(double mean, double std) {
  // Rand.cpp:14-16: scale and shift one standard normal draw.
  return (Rand::real_normal() * std) + mean;
}

double Rand::real_uniform() { return logged(dis_uniform(generator), TAPE_UNIFORM); }

double Rand::real_uniform(double max) { return Rand::real_uniform() * max; }

double Rand::real_uniform(double min, double max) {
  return Rand::real_uniform() * (max - min) + min;
}

double Rand::real_chisquared(unsigned n) {
  dis_chisquared.param(chi_squared_distribution<double>::param_type(n));
  return logged(dis_chisquared(generator), TAPE_CHISQ);
}

double Rand::real_gamma(double a, double b) {
  dis_gamma.param(gamma_distribution<double>::param_type(a, b));
  return logged(dis_gamma(generator), TAPE_GAMMA);
}

extern "C" {
void rand_tape_enable(int on) { g_tape_on = on != 0; }
void rand_tape_clear(void) { g_tape.clear(); }
long rand_tape_size(void) { return static_cast<long>(g_tape.size()); }
void rand_tape_copy(double* values, int* kinds, long n) {
  for (long i = 0; i < n && i < static_cast<long>(g_tape.size()); ++i) {
    values[i] = g_tape[i].value;
    kinds[i] = g_tape[i].kind;
  }
}
void rand_tape_reseed(unsigned long long seed) {
  g_pending_seed = seed;
  Rand::init();
}
}
