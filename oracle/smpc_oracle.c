/*
 * smpc_oracle.c -- CPU restatement of the StarPolymersMD MD/MPC step.
 * TEST INFRASTRUCTURE ONLY (see smpc_oracle.h). Build with -ffp-contract=off:
 * every expression below is written in the reference's evaluation order and
 * must not be fused.
 *
 * Philox stream layout (restated independently of the CUDA code):
 *   key            = { lo32(seed), hi32(seed) }
 *   block(c,s,k)   = Philox4x32-10(ctr = { c, lo32(s), hi32(s), k }, key)  -> w0..w3
 *   U53(lo,hi)     = ((hi:lo) >> 11) * 2^-53 + 2^-54            (open interval)
 *   uA = U53(w0,w1), uB = U53(w2,w3)
 *   cell c, collision s:  block(c,s,0) -> u_phi = uA, u_theta = uB
 *   gamma for cell c:     iteration i uses block(c,s,1+2i) for a Box-Muller
 *                         normal z = sqrt(-2 ln uA) cos(2 pi uB) and block(c,s,2+2i)
 *                         for the acceptance uniform uA (Marsaglia & Tsang 2000)
 *   grid shift:           c = 0xFFFFFFFF: block(c,s,0) -> (uA-1/2, uB-1/2),
 *                         block(c,s,1) -> uA-1/2 for z
 * Philox4x32-10 is Salmon et al., "Parallel random numbers: as easy as 1, 2,
 * 3" (SC'11): multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments
 * 0x9E3779B9 / 0xBB67AE85, ten rounds.
 */
#include "smpc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

struct smpc_orc {
  orc_params p;
  double delrx;
  int shear_on;
  double rot_c, rot_s;
  unsigned n_cell; /* NumberOfCells + 1 */

  long n_f;
  double* fx; /* [3*n_f] */
  double* fv;

  int n_m;
  double* mx;
  double* mv;
  double* mf;
  double* mxv; /* VerletPosition */
  double* mm;  /* mass */
  unsigned char* amphi;
  unsigned char* anchor;
  int n_mol;
  int* mol_start;

  int n_bond;
  int* bsrc;
  int* bdst;
  int* bond_first; /* CSR over source monomer: [n_m+1] */

  /* Verlet lists: CSR in the reference's list order */
  int* vl_start;
  int* vl_idx;
  long vl_cap;
  double com_pos[3];
  double com_vel[3];
  int cs[3];      /* Box::CellSize */
  double csl[3];  /* Box::CellSideLength */
  int* vcell_head; /* per Verlet cell: head of a singly linked list */
  long vcell_cap;
  double grid_lo[3]; /* non-reference presets: grid origin (bounding box) */
  int* vcell_next;
  int verlet_rebuilds;
  double* epot_mol;

  /* MPC cell lists */
  unsigned* c_tot;
  unsigned* c_fl;
  unsigned* c_start;
  long* c_mem; /* >= 0 fluid index, < 0: -(m+1) monomer index */
  int* m_img;  /* Lees-Edwards image index of each monomer when binned wrapped */

  int rng_mode;
  int f32_uniforms; /* orc_set_f32_uniforms: collision draws from 23-bit uniforms */
  const double* inj_shift;
  const double* inj_gamma;
  const double* inj_uphi;
  const double* inj_utheta;
  uint64_t seed;
  uint64_t step_ctr;

  /* periodic MD of many molecules (orc_set_periodic_md) */
  int periodic;
  double pmd_h;       /* MPC step the per-substep delrx is extrapolated with */
  int* adj_start;     /* undirected bond lists, per monomer: [n_m + 1] */
  int* adj_idx;
  unsigned char* adj_anchor;
  int pmd_force_grid; /* test hook: take the grid path whatever the size */

  /* Andersen stochastic thermostat (orc_set_andersen) */
  int andersen;
  double andersen_nu;
  uint64_t andersen_seed;
  uint64_t md_step;
  int lowe;          /* Lowe-Andersen pair thermostat (orc_set_lowe_andersen) */
  double lowe_radius;
  int and_staged;     /* orc_stage_andersen: resets of the next step */
  int and_n;
  int* and_idx;
  double* and_vel;

  int err;
};

/* ------------------------------------------------------------------ Philox */

static inline uint32_t mulhilo32(uint32_t a, uint32_t b, uint32_t* hi) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  return (uint32_t)p;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, hi1;
    uint32_t lo0 = mulhilo32(0xD2511F53u, c0, &hi0);
    uint32_t lo1 = mulhilo32(0xCD9E8D57u, c2, &hi1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline double u53(uint32_t lo, uint32_t hi) {
  uint64_t b = (((uint64_t)hi << 32) | (uint64_t)lo) >> 11;
  return (double)b * 0x1.0p-53 + 0x1.0p-54;
}

static void philox_block(uint64_t seed, uint32_t cell, uint64_t step, uint32_t k, double* uA,
                         double* uB) {
  uint32_t ctr[4] = {cell, (uint32_t)step, (uint32_t)(step >> 32), k};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t w[4];
  orc_philox4x32_10(ctr, key, w);
  *uA = u53(w[0], w[1]);
  if (uB) *uB = u53(w[2], w[3]);
}

/* The FP32 path's uniforms: the top 23 bits of the high word of each pair,
 * (w >> 9) 2^-23 + 2^-24, exact in a float and in a double. */
static inline double u23(uint32_t hi) { return (double)(hi >> 9) * 0x1.0p-23 + 0x1.0p-24; }

static void philox_block23(uint64_t seed, uint32_t cell, uint64_t step, uint32_t k, double* uA,
                           double* uB) {
  uint32_t ctr[4] = {cell, (uint32_t)step, (uint32_t)(step >> 32), k};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t w[4];
  orc_philox4x32_10(ctr, key, w);
  *uA = u23(w[1]);
  if (uB) *uB = u23(w[3]);
}

static double philox_gamma_mode(uint64_t seed, uint64_t step, uint32_t cell, double shape,
                                int f32u) {
  const double d = shape - 1.0 / 3.0;
  const double c = 1.0 / sqrt(9.0 * d);
  void (*block)(uint64_t, uint32_t, uint64_t, uint32_t, double*, double*) =
      f32u ? philox_block23 : philox_block;
  for (uint32_t it = 0; it < 64; ++it) {
    double a, b, u;
    block(seed, cell, step, 1u + 2u * it, &a, &b);
    const double x = sqrt(-2.0 * log(a)) * cos(2.0 * M_PI * b);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    block(seed, cell, step, 2u + 2u * it, &u, NULL);
    const double x2 = x * x;
    if (u < 1.0 - 0.0331 * (x2 * x2)) return d * v;
    if (log(u) < 0.5 * x2 + d * (1.0 - v + log(v))) return d * v;
  }
  return d;
}

double orc_philox_gamma(uint64_t seed, uint64_t step, uint32_t cell, double shape) {
  const double d = shape - 1.0 / 3.0;
  const double c = 1.0 / sqrt(9.0 * d);
  for (uint32_t it = 0; it < 64; ++it) {
    double a, b, u;
    philox_block(seed, cell, step, 1u + 2u * it, &a, &b);
    const double x = sqrt(-2.0 * log(a)) * cos(2.0 * M_PI * b);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    philox_block(seed, cell, step, 2u + 2u * it, &u, NULL);
    const double x2 = x * x;
    if (u < 1.0 - 0.0331 * (x2 * x2)) return d * v;
    if (log(u) < 0.5 * x2 + d * (1.0 - v + log(v))) return d * v;
  }
  return d;
}

/* --------------------------------------------------------------- potentials
 * Potentials.h:14-120, evaluation order kept. */

static inline double fene_force(double r2) { return -30.0 / (1.0 - (r2 / 2.25)); }
static inline double fene_anchor_force(double r2) { return -30.0 / (1.0 - (r2 / 20.25)); }
static inline double fene_pot(double r2) { return -15.0 * 2.25 * log(1.0 - r2 / 2.25); }
static inline double fene_anchor_pot(double r2) { return -15.0 * 20.25 * log(1.0 - r2 / 20.25); }

static inline double aa_force(double r2) {
  double force = 0.0;
  if (r2 < 1.0594631) {
    double rm2 = 1.0 / r2;
    double rm24 = rm2 * rm2 * rm2;
    rm24 *= rm24;
    rm24 *= rm24;
    force = 192.0 * rm2 * rm24 * (rm24 - 0.5);
  }
  return force;
}

static inline double aa_pot(double r2) {
  double pot = 0.0;
  if (r2 < 1.0594631) {
    double rm24 = 1.0 / r2;
    rm24 *= rm24 * rm24;
    rm24 *= rm24;
    rm24 *= rm24;
    pot = 4.0 * rm24 * (rm24 - 1.0) + 1.0;
  }
  return pot;
}

static inline double bb_force(double r2, double lambda) {
  double force = 0.0;
  if (r2 < 1.0594631) {
    double rm2 = 1.0 / r2;
    double rm24 = rm2 * rm2 * rm2;
    rm24 *= rm24;
    rm24 *= rm24;
    force = 192.0 * rm2 * rm24 * (rm24 - 0.5);
  } else if (r2 < 2.25) {
    double rm2 = 1.0 / r2;
    double rm24 = rm2 * rm2 * rm2;
    rm24 *= rm24;
    rm24 *= rm24;
    force = 192.0 * lambda * rm2 * rm24 * (rm24 - 0.5);
  }
  return force;
}

static inline double bb_pot(double r2, double lambda) {
  double pot = 0.0;
  if (r2 < 1.0594631) {
    double rm24 = 1.0 / r2;
    rm24 *= rm24 * rm24;
    rm24 *= rm24;
    rm24 *= rm24;
    pot = 4.0 * rm24 * (rm24 - 1.0) + 1.0 - lambda;
  } else if (r2 < 2.25) {
    double rm24 = 1.0 / r2;
    rm24 *= rm24 * rm24;
    rm24 *= rm24;
    rm24 *= rm24;
    pot = 4.0 * lambda * (rm24 * (rm24 - 1.0) - 0.0000593);
  }
  return pot;
}

/* 12-6 preset used by the benchmark configurations: WCA core (r_c = 2^(1/6))
 * for every pair, plus lambda-scaled LJ attraction out to r = 2.5 for BB pairs
 * (potential shifted to zero at 2.5). Same functional form as the reference's
 * 48-24 pair (Potentials.h:57-120) with exponents 12/6. */
static inline double lj_force_core(double r2) {
  double rm2 = 1.0 / r2;
  double rm6 = rm2 * rm2 * rm2;
  return 48.0 * rm2 * rm6 * (rm6 - 0.5);
}
static inline double lj_pot_core(double r2) {
  double rm6 = 1.0 / r2;
  rm6 *= rm6 * rm6;
  return 4.0 * rm6 * (rm6 - 1.0);
}
#define LJ126_RC2_REP 1.2599210498948732 /* 2^(1/3) */
#define LJ126_RC2_ATT 6.25
#define LJ126_SHIFT (-0.016316891136)    /* 4 (2.5^-12 - 2.5^-6) */

static inline double pair_force(int pot, int bb, double r2, double lambda) {
  if (pot == ORC_POT_REF4824) return bb ? bb_force(r2, lambda) : aa_force(r2);
  if (r2 < LJ126_RC2_REP) return lj_force_core(r2);
  if (bb && r2 < LJ126_RC2_ATT) return lambda * lj_force_core(r2);
  return 0.0;
}
static inline double pair_pot(int pot, int bb, double r2, double lambda) {
  if (pot == ORC_POT_REF4824) return bb ? bb_pot(r2, lambda) : aa_pot(r2);
  if (r2 < LJ126_RC2_REP) return lj_pot_core(r2) + 1.0 - (bb ? lambda : 0.0);
  if (bb && r2 < LJ126_RC2_ATT) return lambda * (lj_pot_core(r2) - LJ126_SHIFT);
  return 0.0;
}

/* ------------------------------------------------------------------ set-up */

smpc_orc* orc_create(const orc_params* p, long n_fluid, int n_mono, int n_mol,
                     const int* mol_start) {
  smpc_orc* o = (smpc_orc*)calloc(1, sizeof(smpc_orc));
  if (!o) return NULL;
  o->p = *p;
  o->shear_on = (p->shear != 0.0);
  o->rot_c = cos(130.0 * M_PI / 180.0); /* MPC.cpp:23-24 */
  o->rot_s = sin(130.0 * M_PI / 180.0);
  o->n_cell = (unsigned)(p->L[0] * p->L[1] * p->L[2]);
  o->n_f = n_fluid;
  o->n_m = n_mono;
  o->fx = (double*)calloc((size_t)(3 * n_fluid + 3), sizeof(double));
  o->fv = (double*)calloc((size_t)(3 * n_fluid + 3), sizeof(double));
  size_t m3 = (size_t)(3 * n_mono + 3);
  o->mx = (double*)calloc(m3, sizeof(double));
  o->mv = (double*)calloc(m3, sizeof(double));
  o->mf = (double*)calloc(m3, sizeof(double));
  o->mxv = (double*)calloc(m3, sizeof(double));
  o->mm = (double*)calloc((size_t)n_mono + 1, sizeof(double));
  o->amphi = (unsigned char*)calloc((size_t)n_mono + 1, 1);
  o->anchor = (unsigned char*)calloc((size_t)n_mono + 1, 1);
  o->n_mol = n_mol;
  o->mol_start = (int*)calloc((size_t)n_mol + 1, sizeof(int));
  if (mol_start) memcpy(o->mol_start, mol_start, sizeof(int) * (size_t)(n_mol + 1));
  o->epot_mol = (double*)calloc((size_t)n_mol + 1, sizeof(double));
  o->vl_start = (int*)calloc((size_t)n_mono + 1, sizeof(int));
  o->vl_cap = 64L * (n_mono + 1);
  o->vl_idx = (int*)malloc(sizeof(int) * (size_t)o->vl_cap);
  o->vcell_next = (int*)malloc(sizeof(int) * (size_t)(n_mono + 1));
  o->bond_first = (int*)calloc((size_t)n_mono + 2, sizeof(int));
  /* Box.cpp:20-25: Verlet cell grid of int(L/VerletRadius) cells per axis. */
  long ncv = 1;
  for (int d = 0; d < 3; ++d) {
    o->cs[d] = (int)(p->L[d] / 2.0);
    if (o->cs[d] < 1) o->cs[d] = 1;
    o->csl[d] = p->L[d] / (double)o->cs[d];
    ncv *= o->cs[d];
  }
  o->vcell_head = (int*)malloc(sizeof(int) * (size_t)ncv);
  o->vcell_cap = ncv;
  o->c_tot = (unsigned*)calloc(o->n_cell, sizeof(unsigned));
  o->c_fl = (unsigned*)calloc(o->n_cell, sizeof(unsigned));
  o->c_start = (unsigned*)calloc((size_t)o->n_cell + 1, sizeof(unsigned));
  o->c_mem = (long*)malloc(sizeof(long) * (size_t)(n_fluid + n_mono + 1));
  o->m_img = (int*)calloc((size_t)n_mono + 1, sizeof(int));
  if (!o->fx || !o->fv || !o->mx || !o->vl_idx || !o->vcell_head || !o->c_mem) o->err |= ORC_ERR_ALLOC;
  o->rng_mode = ORC_RNG_INJECT;
  return o;
}

void orc_destroy(smpc_orc* o) {
  if (!o) return;
  free(o->fx); free(o->fv); free(o->mx); free(o->mv); free(o->mf); free(o->mxv); free(o->mm);
  free(o->amphi); free(o->anchor); free(o->mol_start); free(o->epot_mol);
  free(o->bsrc); free(o->bdst); free(o->bond_first); free(o->vl_start); free(o->vl_idx);
  free(o->vcell_head); free(o->vcell_next); free(o->c_tot); free(o->c_fl); free(o->c_start);
  free(o->c_mem);
  free(o->m_img);
  free(o->adj_start); free(o->adj_idx); free(o->adj_anchor);
  free(o->and_idx); free(o->and_vel);
  free(o);
}

int orc_error(const smpc_orc* o) { return o->err; }
void orc_clear_error(smpc_orc* o) { o->err = 0; }

void orc_set_fluid(smpc_orc* o, const double* pos, const double* vel) {
  memcpy(o->fx, pos, sizeof(double) * 3 * (size_t)o->n_f);
  memcpy(o->fv, vel, sizeof(double) * 3 * (size_t)o->n_f);
}
void orc_get_fluid(const smpc_orc* o, double* pos, double* vel) {
  if (pos) memcpy(pos, o->fx, sizeof(double) * 3 * (size_t)o->n_f);
  if (vel) memcpy(vel, o->fv, sizeof(double) * 3 * (size_t)o->n_f);
}

void orc_set_monomers(smpc_orc* o, const double* pos, const double* vel, const double* force,
                      const double* mass, const int* amphi, const int* anchor) {
  size_t n3 = sizeof(double) * 3 * (size_t)o->n_m;
  if (pos) memcpy(o->mx, pos, n3);
  if (vel) memcpy(o->mv, vel, n3);
  if (force) memcpy(o->mf, force, n3);
  for (int i = 0; i < o->n_m; ++i) {
    if (mass) o->mm[i] = mass[i];
    if (amphi) o->amphi[i] = (unsigned char)(amphi[i] != 0);
    if (anchor) o->anchor[i] = (unsigned char)(anchor[i] != 0);
  }
}

void orc_get_monomers(const smpc_orc* o, double* pos, double* vel, double* force) {
  size_t n3 = sizeof(double) * 3 * (size_t)o->n_m;
  if (pos) memcpy(pos, o->mx, n3);
  if (vel) memcpy(vel, o->mv, n3);
  if (force) memcpy(force, o->mf, n3);
}

void orc_set_bonds(smpc_orc* o, int n_bond, const int* src, const int* dst) {
  free(o->bsrc);
  free(o->bdst);
  o->n_bond = n_bond;
  o->bsrc = (int*)malloc(sizeof(int) * (size_t)(n_bond + 1));
  o->bdst = (int*)malloc(sizeof(int) * (size_t)(n_bond + 1));
  memset(o->bond_first, 0, sizeof(int) * (size_t)(o->n_m + 2));
  /* Bonds arrive grouped by source monomer in Neighbors order. */
  for (int b = 0; b < n_bond; ++b) {
    o->bsrc[b] = src[b];
    o->bdst[b] = dst[b];
    o->bond_first[src[b] + 1]++;
  }
  for (int i = 0; i < o->n_m; ++i) o->bond_first[i + 1] += o->bond_first[i];
}

double orc_delrx(const smpc_orc* o) { return o->delrx; }
void orc_set_delrx(smpc_orc* o, double d) { o->delrx = d; }

void orc_set_inject(smpc_orc* o, const double* shift3, const double* gamma, const double* u_phi,
                    const double* u_theta) {
  o->rng_mode = ORC_RNG_INJECT;
  o->inj_shift = shift3;
  o->inj_gamma = gamma;
  o->inj_uphi = u_phi;
  o->inj_utheta = u_theta;
}

void orc_set_philox(smpc_orc* o, uint64_t seed, uint64_t collision_counter) {
  o->rng_mode = ORC_RNG_PHILOX;
  o->seed = seed;
  o->step_ctr = collision_counter;
}
uint64_t orc_collision_counter(const smpc_orc* o) { return o->step_ctr; }
void orc_set_f32_uniforms(smpc_orc* o, int on) { o->f32_uniforms = on != 0; }

/* -------------------------------------------------------- Box: Verlet/MD */

/* Box::center_of_mass_reference_frame (Box.cpp:81-102): only the COM of
 * molecule 0 is kept (COM_Pos / COM_Vel). */
static void com_frame(smpc_orc* o) {
  if (o->n_mol < 1) return;
  double c[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
  int b = o->mol_start[0], e = o->mol_start[1];
  for (int i = b; i < e; ++i) {
    for (int d = 0; d < 3; ++d) {
      c[d] += o->mx[3 * i + d];
      cv[d] += o->mv[3 * i + d];
    }
  }
  unsigned n = (unsigned)(e - b);
  for (int d = 0; d < 3; ++d) {
    o->com_pos[d] = c[d] / n;
    o->com_vel[d] = cv[d] / n;
  }
}

static inline int vcell_of(const smpc_orc* o, int i, int* cn) {
  if (o->p.potential != ORC_POT_REF4824) {
    for (int d = 0; d < 3; ++d) cn[d] = (int)((o->mx[3 * i + d] - o->grid_lo[d]) / o->csl[d]);
  } else {
    for (int d = 0; d < 3; ++d)
      cn[d] = (int)((o->mx[3 * i + d] - o->com_pos[d] + o->p.L[d] * 0.5) / o->csl[d]);
  }
  return !(cn[0] < 0 || cn[0] >= o->cs[0] || cn[1] < 0 || cn[1] >= o->cs[1] || cn[2] < 0 ||
           cn[2] >= o->cs[2]);
}

/* Box::update_VerletLists (Box.cpp:105-180). Cell contents are forward_lists
 * filled with push_front and each VerletList is filled with push_front, so
 * the final list order is the reverse of the traversal order; that order is
 * reproduced here so force sums match bit for bit. */
static void update_verlet(smpc_orc* o) {
  o->verlet_rebuilds++;
  const int n = o->n_m;
  com_frame(o);
  if (o->p.potential != ORC_POT_REF4824 && n > 0) {
    /* cells of side >= r_verlet over the monomers' bounding box */
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) lo[d] = hi[d] = o->mx[d];
    for (int i = 1; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
        if (o->mx[3 * i + d] < lo[d]) lo[d] = o->mx[3 * i + d];
        if (o->mx[3 * i + d] > hi[d]) hi[d] = o->mx[3 * i + d];
      }
    long need = 1;
    for (int d = 0; d < 3; ++d) {
      o->grid_lo[d] = lo[d] - 1e-6;
      double ext = hi[d] - lo[d] + 2e-6;
      o->cs[d] = (int)(ext / o->p.r_verlet);
      if (o->cs[d] < 1) o->cs[d] = 1;
      o->csl[d] = ext / o->cs[d];
      if (o->csl[d] < o->p.r_verlet) { o->cs[d] = o->cs[d] > 1 ? o->cs[d] - 1 : 1; o->csl[d] = ext / o->cs[d]; }
      need *= o->cs[d];
    }
    if (need > o->vcell_cap) {
      o->vcell_head = (int*)realloc(o->vcell_head, sizeof(int) * (size_t)need);
      o->vcell_cap = need;
    }
  }
  const long ncv = (long)o->cs[0] * o->cs[1] * o->cs[2];
  for (long c = 0; c < ncv; ++c) o->vcell_head[c] = -1;
  int cn[3];
  for (int i = 0; i < n; ++i) {
    if (!vcell_of(o, i, cn)) {
      o->err |= ORC_ERR_VERLET_CELL;
      continue;
    }
    for (int d = 0; d < 3; ++d) o->mxv[3 * i + d] = o->mx[3 * i + d];
    long c = ((long)cn[0] * o->cs[1] + cn[1]) * o->cs[2] + cn[2];
    o->vcell_next[i] = o->vcell_head[c]; /* push_front */
    o->vcell_head[c] = i;
  }
  const double rv2 = o->p.r_verlet * o->p.r_verlet;
  long fill = 0;
  int* tmp = (int*)malloc(sizeof(int) * (size_t)(n + 1));
  for (int i = 0; i < n; ++i) {
    o->vl_start[i] = (int)fill;
    int cnt = 0;
    if (vcell_of(o, i, cn)) {
      for (int j = cn[0] - 1; j < cn[0] + 2; ++j) {
        if (j < 0 || j >= o->cs[0]) continue;
        for (int k = cn[1] - 1; k < cn[1] + 2; ++k) {
          if (k < 0 || k >= o->cs[1]) continue;
          for (int l = cn[2] - 1; l < cn[2] + 2; ++l) {
            if (l < 0 || l >= o->cs[2]) continue;
            long c = ((long)j * o->cs[1] + k) * o->cs[2] + l;
            for (int q = o->vcell_head[c]; q >= 0; q = o->vcell_next[q]) {
              if (q == i) continue;
              double dx = o->mx[3 * q] - o->mx[3 * i];
              double dy = o->mx[3 * q + 1] - o->mx[3 * i + 1];
              double dz = o->mx[3 * q + 2] - o->mx[3 * i + 2];
              double r2 = (dx * dx + dy * dy) + dz * dz;
              if (r2 <= rv2) tmp[cnt++] = q;
            }
          }
        }
      }
    }
    if (fill + cnt > o->vl_cap) {
      o->vl_cap = 2 * (fill + cnt) + 64;
      o->vl_idx = (int*)realloc(o->vl_idx, sizeof(int) * (size_t)o->vl_cap);
    }
    for (int t = cnt - 1; t >= 0; --t) o->vl_idx[fill++] = tmp[t]; /* push_front order */
  }
  o->vl_start[n] = (int)fill;
  free(tmp);
}

/* Box::check_VerletLists (Box.cpp:182-194). */
static void check_verlet(smpc_orc* o) {
  const double lim = (o->p.r_verlet - o->p.r_cut) * 0.5;
  for (int i = 0; i < o->n_m; ++i) {
    double dx = o->mx[3 * i] - o->mxv[3 * i];
    double dy = o->mx[3 * i + 1] - o->mxv[3 * i + 1];
    double dz = o->mx[3 * i + 2] - o->mxv[3 * i + 2];
    if (sqrt((dx * dx + dy * dy) + dz * dz) > lim) {
      update_verlet(o);
      return;
    }
  }
}

/* Box::calculate_forces_verlet (Box.cpp:243-286). */
static void forces_verlet(smpc_orc* o, int calc_epot) {
  for (int m = 0; m < o->n_mol; ++m) o->epot_mol[m] = 0.0;
  for (int i = 0; i < 3 * o->n_m; ++i) o->mf[i] = o->mf[i] * 0.0;
  const double lambda = o->p.lambda;
  const int pot = o->p.potential;
  for (int m = 0; m < o->n_mol; ++m) {
    double ep = 0.0;
    for (int i = o->mol_start[m]; i < o->mol_start[m + 1]; ++i) {
      double* fi = o->mf + 3 * i;
      const double* xi = o->mx + 3 * i;
      for (int t = o->vl_start[i]; t < o->vl_start[i + 1]; ++t) {
        const int j = o->vl_idx[t];
        const double* xj = o->mx + 3 * j;
        double d0 = xj[0] - xi[0], d1 = xj[1] - xi[1], d2 = xj[2] - xi[2];
        double r2 = (d0 * d0 + d1 * d1) + d2 * d2;
        int bb = (o->amphi[i] == 1 && o->amphi[j] == 1);
        if (calc_epot) ep += 0.5 * pair_pot(pot, bb, r2, lambda);
        double fa = pair_force(pot, bb, r2, lambda);
        fi[0] -= d0 * fa;
        fi[1] -= d1 * fa;
        fi[2] -= d2 * fa;
      }
      for (int b = o->bond_first[i]; b < o->bond_first[i + 1]; ++b) {
        const int j = o->bdst[b];
        const double* xj = o->mx + 3 * j;
        double d0 = xj[0] - xi[0], d1 = xj[1] - xi[1], d2 = xj[2] - xi[2];
        double r2 = (d0 * d0 + d1 * d1) + d2 * d2;
        double fa;
        if (pot != ORC_POT_REF4824) {
          /* 12-6 preset: FENE argument capped at 0.98 R0^2 (finite, restoring) */
          const double cap = (o->anchor[i] ? 20.25 : 2.25) * 0.98;
          if (r2 > cap) r2 = cap;
        }
        if (o->anchor[i]) {
          if (calc_epot) ep += fene_anchor_pot(r2);
          fa = fene_anchor_force(r2);
        } else {
          if (calc_epot) ep += fene_pot(r2);
          fa = fene_force(r2);
        }
        double f0 = d0 * fa, f1 = d1 * fa, f2 = d2 * fa;
        fi[0] -= f0;
        fi[1] -= f1;
        fi[2] -= f2;
        o->mf[3 * j] += f0;
        o->mf[3 * j + 1] += f1;
        o->mf[3 * j + 2] += f2;
      }
    }
    o->epot_mol[m] = ep;
  }
}

static void pmd_init(smpc_orc* o);

void orc_init_md(smpc_orc* o) {
  if (o->periodic) {
    pmd_init(o);
    return;
  }
  update_verlet(o);
  forces_verlet(o, 0);
}

/* Thermostat_None::propagate (Thermostat_None.cpp:21-38). */
/* AndersenStochastic::propagate (Andersen_stochastic.cpp:30-59): the kick is
 * grouped as F (dt/2 / m); after the second kick each monomer, with
 * probability nu dt, gets every velocity component from N(0, sqrt(kT / m)).
 * Draws restated from the GPU's layout: Philox on the seed, counter
 * (0x80000000 | monomer, MD step, k); k = 0: trigger, u1; k = 1: u2, u3;
 * k = 2: u4; Box-Muller (u1, u2) -> x, y and (u3, u4) -> z. */
void orc_set_andersen(smpc_orc* o, double nu, uint64_t seed) {
  o->andersen = 1;
  o->andersen_nu = nu;
  o->andersen_seed = seed;
}

/* Injected resets (the reference's own Rand draws, decoded on the host:
 * Andersen_stochastic.cpp:49-58) replace the Philox draws of the next step. */
void orc_stage_andersen(smpc_orc* o, int n, const int* idx, const double* vel) {
  free(o->and_idx);
  free(o->and_vel);
  o->and_idx = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  o->and_vel = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  for (int k = 0; k < n; ++k) {
    o->and_idx[k] = idx[k];
    for (int d = 0; d < 3; ++d) o->and_vel[3 * k + d] = vel[3 * k + d];
  }
  o->and_n = n;
  o->and_staged = 1;
}

static inline double md_kick(const smpc_orc* o, double f, double m, double dth) {
  return o->andersen ? f * (dth / m) : (f / m) * dth;
}

static void andersen_step(smpc_orc* o) {
  if (o->and_staged) {
    for (int k = 0; k < o->and_n; ++k)
      for (int d = 0; d < 3; ++d) o->mv[3 * o->and_idx[k] + d] = o->and_vel[3 * k + d];
    o->and_staged = 0;
    return;
  }
  const double p = o->andersen_nu * o->p.md_dt;
  const double sigma = sqrt(o->p.kT);
  for (int i = 0; i < o->n_m; ++i) {
    const uint32_t c = 0x80000000u | (uint32_t)i;
    double t, u1, u2, u3, u4;
    philox_block(o->andersen_seed, c, o->md_step, 0u, &t, &u1);
    if (!(t < p)) continue;
    philox_block(o->andersen_seed, c, o->md_step, 1u, &u2, &u3);
    philox_block(o->andersen_seed, c, o->md_step, 2u, &u4, NULL);
    const double s = sigma / sqrt(o->mm[i]);
    const double r1 = sqrt(-2.0 * log(u1)), r2 = sqrt(-2.0 * log(u3));
    const double two_pi = 6.283185307179586476925286766559;
    o->mv[3 * i] = s * (r1 * cos(two_pi * u2));
    o->mv[3 * i + 1] = s * (r1 * sin(two_pi * u2));
    o->mv[3 * i + 2] = s * (r2 * cos(two_pi * u4));
  }
}

/* Lowe-Andersen (Lowe_Andersen.cpp:46-88): after the forces, every Verlet-list
 * candidate (i, j) closer than the radius collides with probability
 * nu dt exp(-nu dt) / 2; collisions one after another on the updated
 * velocities, beads i ascending and partners j ascending. Draws restated from
 * the GPU's layout: Philox on the seed, counter (0x40000000 | i, MD step,
 * 2 j + k); k = 0: trigger, u1; k = 1: u2; z = sqrt(-2 ln u1) cos(2 pi u2).
 * The pair arithmetic is Lowe_Andersen::collide (Lowe_Andersen.cpp:28-41). */
void orc_set_lowe_andersen(smpc_orc* o, double nu, double radius, uint64_t seed) {
  o->lowe = 1;
  o->andersen_nu = nu;
  o->lowe_radius = radius;
  o->andersen_seed = seed;
}

static int lowe_cmp_int(const void* a, const void* b) {
  const int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

static void lowe_step(smpc_orc* o) {
  const double nudt = o->andersen_nu * o->p.md_dt * exp(-o->p.md_dt * o->andersen_nu);
  const double half = nudt * 0.5;
  const double two_pi = 6.283185307179586476925286766559;
  int cap = 0;
  int* js = NULL;
  for (int i = 0; i < o->n_m; ++i) {
    const int a = o->vl_start[i], b = o->vl_start[i + 1];
    if (b - a > cap) {
      cap = b - a;
      js = (int*)realloc(js, sizeof(int) * (size_t)cap);
    }
    for (int t = a; t < b; ++t) js[t - a] = o->vl_idx[t];
    qsort(js, (size_t)(b - a), sizeof(int), lowe_cmp_int);
    const uint32_t c = 0x40000000u | (uint32_t)i;
    for (int q = 0; q < b - a; ++q) {
      const int j = js[q];
      double tr, u1, u2;
      philox_block(o->andersen_seed, c, o->md_step, 2u * (uint32_t)j, &tr, &u1);
      if (half < tr) continue;
      const double* xi = o->mx + 3 * i;
      const double* xj = o->mx + 3 * j;
      const double d0 = xj[0] - xi[0], d1 = xj[1] - xi[1], d2 = xj[2] - xi[2];
      const double dist = sqrt((d0 * d0 + d1 * d1) + d2 * d2);
      if (!(dist < o->lowe_radius)) continue;
      philox_block(o->andersen_seed, c, o->md_step, 2u * (uint32_t)j + 1u, &u2, NULL);
      const double mi = o->mm[i], mj = o->mm[j];
      const double mu = mi == mj ? 0.5 * mi : mi * mj / (mi + mj);
      const double sigma = sqrt(o->p.kT / mu);
      const double z = sqrt(-2.0 * log(u1)) * cos(two_pi * u2);
      const double e0 = d0 / dist, e1 = d1 / dist, e2 = d2 / dist;
      const double tv = sigma * z, ci = mu / mi, cj = mu / mj;
      double* vi = o->mv + 3 * i;
      double* vj = o->mv + 3 * j;
      const double w0 = vj[0] - vi[0], w1 = vj[1] - vi[1], w2 = vj[2] - vi[2];
      const double sc = tv + ((w0 * e0 + w1 * e1) + w2 * e2);
      const double dv0 = e0 * sc, dv1 = e1 * sc, dv2 = e2 * sc;
      vi[0] += dv0 * ci;
      vi[1] += dv1 * ci;
      vi[2] += dv2 * ci;
      vj[0] -= dv0 * cj;
      vj[1] -= dv1 * cj;
      vj[2] -= dv2 * cj;
    }
  }
  free(js);
}

static void pmd_propagate(smpc_orc* o, int calc_epot);

void orc_propagate(smpc_orc* o, int calc_epot) {
  if (o->periodic) {
    pmd_propagate(o, calc_epot);
    return;
  }
  const double dt = o->p.md_dt;
  const double dth = dt * 0.50;
  for (int i = 0; i < o->n_m; ++i) {
    for (int d = 0; d < 3; ++d) {
      o->mv[3 * i + d] += md_kick(o, o->mf[3 * i + d], o->mm[i], dth);
      o->mx[3 * i + d] += o->mv[3 * i + d] * dt;
    }
  }
  check_verlet(o);
  forces_verlet(o, calc_epot);
  if (o->lowe) lowe_step(o);
  for (int i = 0; i < o->n_m; ++i)
    for (int d = 0; d < 3; ++d) o->mv[3 * i + d] += md_kick(o, o->mf[3 * i + d], o->mm[i], dth);
  if (o->andersen) andersen_step(o);
  o->md_step++;
}

double orc_epot(const smpc_orc* o) {
  double e = 0.0;
  for (int m = 0; m < o->n_mol; ++m) e += o->epot_mol[m];
  return e;
}

int orc_verlet_rebuilds(const smpc_orc* o) { return o->verlet_rebuilds; }

/* ----------------------------------------------------------------- MPC */

/* MPC::LEBC (MPC.cpp:421-429) and MPC::wrap(Particle&) (MPC.cpp:487-490). */
static inline void wrap_particle(const smpc_orc* o, double* x, double* v) {
  const double Lx = o->p.L[0], Ly = o->p.L[1], Lz = o->p.L[2];
  if (o->shear_on) {
    double cy = round(x[1] / Ly);
    x[0] -= Lx * round(x[0] / Lx);
    x[0] -= cy * o->delrx;
    x[0] -= Lx * round(x[0] / Lx);
    x[1] -= Ly * cy;
    x[2] -= Lz * round(x[2] / Lz);
    v[0] -= cy * o->p.shear * Ly;
  } else {
    x[0] -= round(x[0] / Lx) * Lx;
    x[1] -= round(x[1] / Ly) * Ly;
    x[2] -= round(x[2] / Lz) * Lz;
  }
}

/* MPC::check_bounds (MPC.cpp:160-190). */
static void check_bounds(smpc_orc* o) {
  if (o->periodic) return; /* no recentring in a periodic box */
  int out = 0;
  for (int i = 0; i < o->n_m && !out; ++i)
    for (int d = 0; d < 3; ++d)
      if (fabs(o->mx[3 * i + d]) >= (o->p.L[d] * 0.5 - 0.5)) {
        out = 1;
        break;
      }
  if (!out || o->n_mol < 1) return;
  double com[3] = {0, 0, 0}, comv[3] = {0, 0, 0};
  int b = o->mol_start[0], e = o->mol_start[1];
  for (int i = b; i < e; ++i)
    for (int d = 0; d < 3; ++d) {
      com[d] += o->mx[3 * i + d];
      comv[d] += o->mv[3 * i + d];
    }
  unsigned n = (unsigned)(e - b);
  for (int d = 0; d < 3; ++d) {
    com[d] /= n;
    comv[d] /= n;
  }
  for (int i = 0; i < o->n_m; ++i)
    for (int d = 0; d < 3; ++d) {
      o->mx[3 * i + d] -= com[d];
      o->mv[3 * i + d] -= comv[d];
    }
  for (long i = 0; i < o->n_f; ++i) {
    for (int d = 0; d < 3; ++d) {
      o->fx[3 * i + d] -= com[d];
      o->fv[3 * i + d] -= comv[d];
    }
    wrap_particle(o, o->fx + 3 * i, o->fv + 3 * i);
  }
}

/* MPC::sort cell index formula (MPC.cpp:209,225). */
static inline unsigned cell_index(const smpc_orc* o, const double* x) {
  const int Lx = o->p.L[0], Ly = o->p.L[1], Lz = o->p.L[2];
  int c = (int)(x[0] + Lx * 0.5) + Lx * (int)(x[1] + Ly * 0.5) + Lx * Ly * (int)(x[2] + Lz * 0.5);
  return (unsigned)c;
}

/* MPC::sort (MPC.cpp:201-237) as a stable counting sort: per cell, fluid in
 * Fluid order then monomers in molecule order, exactly the push_back order. */
static void mpc_sort(smpc_orc* o) {
  const unsigned nc = o->n_cell;
  const unsigned last = nc - 1; /* NumberOfCells */
  memset(o->c_tot, 0, sizeof(unsigned) * nc);
  memset(o->c_fl, 0, sizeof(unsigned) * nc);
  unsigned* key = (unsigned*)malloc(sizeof(unsigned) * (size_t)(o->n_f + o->n_m + 1));
  for (long i = 0; i < o->n_f; ++i) {
    unsigned c = cell_index(o, o->fx + 3 * i);
    key[i] = c;
    if (c > last) {
      o->err |= ORC_ERR_FLUID_CELL;
      continue;
    }
    o->c_tot[c]++;
    o->c_fl[c]++;
  }
  for (int m = 0; m < o->n_m; ++m) {
    unsigned c;
    if (o->p.mono_wrap) {
      /* bin at the periodic image; clamp faces like the fast path */
      double x[3] = {o->mx[3 * m], o->mx[3 * m + 1], o->mx[3 * m + 2]}, dv = 0.0;
      o->m_img[m] = (int)round(x[1] / o->p.L[1]);
      wrap_particle(o, x, &dv);
      int ci[3];
      for (int d = 0; d < 3; ++d) {
        ci[d] = (int)(x[d] + o->p.L[d] * 0.5);
        if (ci[d] < 0) ci[d] = 0;
        if (ci[d] >= o->p.L[d]) ci[d] = o->p.L[d] - 1;
      }
      c = (unsigned)(ci[0] + o->p.L[0] * (ci[1] + o->p.L[1] * ci[2]));
    } else {
      o->m_img[m] = 0;
      c = cell_index(o, o->mx + 3 * m);
    }
    key[o->n_f + m] = c;
    if (c > last) {
      o->err |= ORC_ERR_MONO_CELL;
      continue;
    }
    o->c_tot[c]++;
  }
  unsigned acc = 0;
  for (unsigned c = 0; c < nc; ++c) {
    o->c_start[c] = acc;
    acc += o->c_tot[c];
  }
  o->c_start[nc] = acc;
  unsigned* fillp = (unsigned*)malloc(sizeof(unsigned) * nc);
  memcpy(fillp, o->c_start, sizeof(unsigned) * nc);
  for (long i = 0; i < o->n_f; ++i)
    if (key[i] <= last) o->c_mem[fillp[key[i]]++] = i;
  for (int m = 0; m < o->n_m; ++m)
    if (key[o->n_f + m] <= last) o->c_mem[fillp[key[o->n_f + m]]++] = -(long)m - 1;
  free(fillp);
  free(key);
}

static inline double* pvel(smpc_orc* o, long id) {
  return id >= 0 ? o->fv + 3 * id : o->mv + 3 * (-id - 1);
}
static inline double pmass(const smpc_orc* o, long id) {
  return id >= 0 ? 1.0 : o->mm[-id - 1];
}

/* MPC::calculateCMV (MPC.cpp:314-322). */
static void cell_cmv(smpc_orc* o, unsigned c, double* cmv) {
  cmv[0] = cmv[1] = cmv[2] = 0.0;
  double tm = 0.0;
  for (unsigned k = o->c_start[c]; k < o->c_start[c + 1]; ++k) {
    long id = o->c_mem[k];
    const double* v = pvel(o, id);
    double m = pmass(o, id);
    cmv[0] += v[0] * m;
    cmv[1] += v[1] * m;
    cmv[2] += v[2] * m;
    tm += m;
  }
  if (tm > 0) {
    cmv[0] /= tm;
    cmv[1] /= tm;
    cmv[2] /= tm;
  }
}

/* MPC::thermostat (MPC.cpp:273-299). */
static void cell_thermostat(smpc_orc* o, unsigned c, const double* cmv) {
  double ekin = 0.0;
  unsigned count = 0;
  for (unsigned k = o->c_start[c]; k < o->c_start[c + 1]; ++k) {
    long id = o->c_mem[k];
    const double* v = pvel(o, id);
    double d0 = v[0] - cmv[0], d1 = v[1] - cmv[1], d2 = v[2] - cmv[2];
    ekin += pmass(o, id) * ((d0 * d0 + d1 * d1) + d2 * d2);
    count++;
  }
  if (count < 2) return;
  ekin *= 0.5;
  double g;
  if (o->rng_mode == ORC_RNG_INJECT) {
    g = o->inj_gamma ? o->inj_gamma[c] * 1.0 : 0.0;
    /* injected values are Gamma(1.5(n-1), kT) variates as drawn */
  } else {
    g = philox_gamma_mode(o->seed, o->step_ctr, c, 1.5 * (count - 1), o->f32_uniforms) * o->p.kT;
  }
  double scaling = sqrt(g / ekin);
  for (unsigned k = o->c_start[c]; k < o->c_start[c + 1]; ++k) {
    double* v = pvel(o, o->c_mem[k]);
    for (int d = 0; d < 3; ++d) v[d] = scaling * v[d] + (1 - scaling) * cmv[d];
  }
}

/* Position of a cell member in the collision frame: the solvent's stored
 * (shifted, wrapped) position; a monomer's shifted position, at its
 * Lees-Edwards image when monomers are binned wrapped. */
static void ppos(const smpc_orc* o, long id, double* x) {
  if (id >= 0) {
    for (int d = 0; d < 3; ++d) x[d] = o->fx[3 * id + d];
    return;
  }
  const int m = (int)(-id - 1);
  for (int d = 0; d < 3; ++d) x[d] = o->mx[3 * m + d];
  if (o->p.mono_wrap) {
    double dv = 0.0;
    wrap_particle(o, x, &dv);
  }
}

/* x = A^-1 b for symmetric positive-definite A by the Cholesky factor
 * A = L L^T, column by column, then forward and back substitution. */
static void llt_solve3(const double A[3][3], const double b[3], double x[3]) {
  double l[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, y[3];
  for (int j = 0; j < 3; ++j) {
    double s = A[j][j];
    for (int k = 0; k < j; ++k) s -= l[j][k] * l[j][k];
    l[j][j] = sqrt(s);
    for (int i = j + 1; i < 3; ++i) {
      double t = A[i][j];
      for (int k = 0; k < j; ++k) t -= l[i][k] * l[j][k];
      l[i][j] = t / l[j][j];
    }
  }
  for (int i = 0; i < 3; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= l[i][k] * y[k];
    y[i] = s / l[i][i];
  }
  for (int i = 2; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < 3; ++k) s -= l[k][i] * x[k];
    x[i] = s / l[i][i];
  }
}

/* MPC::calculateCMP and MPC::calculateAngular (MPC.cpp:324-374): the cell's
 * centre of mass and the angular velocity that restores its angular momentum
 * after the rotation R, in the reference's operation order. */
static void cell_angular(smpc_orc* o, unsigned c, const double* cmv, double R[3][3],
                         double* cmp, double* ang) {
  double tm = 0.0;
  cmp[0] = cmp[1] = cmp[2] = 0.0;
  for (unsigned k = o->c_start[c]; k < o->c_start[c + 1]; ++k) {
    const long id = o->c_mem[k];
    double x[3];
    ppos(o, id, x);
    const double m = pmass(o, id);
    cmp[0] += x[0] * m;
    cmp[1] += x[1] * m;
    cmp[2] += x[2] * m;
    tm += m;
  }
  if (tm > 0) {
    cmp[0] /= tm;
    cmp[1] /= tm;
    cmp[2] /= tm;
  }
  double cv[3] = {0, 0, 0}, I[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (unsigned k = o->c_start[c]; k < o->c_start[c + 1]; ++k) {
    const long id = o->c_mem[k];
    double x[3];
    ppos(o, id, x);
    const double* v = pvel(o, id);
    const double m = pmass(o, id);
    const double q[3] = {x[0] - cmp[0], x[1] - cmp[1], x[2] - cmp[2]};
    const double u[3] = {v[0] - cmv[0], v[1] - cmv[1], v[2] - cmv[2]};
    double w[3];
    for (int i = 0; i < 3; ++i) w[i] = u[i] - ((R[i][0] * u[0] + R[i][1] * u[1]) + R[i][2] * u[2]);
    const double cr[3] = {q[1] * w[2] - q[2] * w[1], q[2] * w[0] - q[0] * w[2],
                          q[0] * w[1] - q[1] * w[0]};
    cv[0] += m * cr[0];
    cv[1] += m * cr[1];
    cv[2] += m * cr[2];
    I[0][0] += m * (q[1] * q[1] + q[2] * q[2]);
    I[1][1] += m * (q[0] * q[0] + q[2] * q[2]);
    I[2][2] += m * (q[1] * q[1] + q[0] * q[0]);
    I[0][1] -= m * q[0] * q[1];
    I[0][2] -= m * q[0] * q[2];
    I[1][2] -= m * q[1] * q[2];
  }
  I[1][0] = I[0][1];
  I[2][0] = I[0][2];
  I[2][1] = I[1][2];
  llt_solve3(I, cv, ang);
}

/* MPC::collide (MPC.cpp:239-270), with the angular-momentum correction in
 * cells of more than two particles when p.angular_momentum is set. */
static void cell_collide(smpc_orc* o, unsigned c, const double* cmv) {
  double uphi, uth;
  if (o->rng_mode == ORC_RNG_INJECT) {
    uphi = o->inj_uphi[c];
    uth = o->inj_utheta[c];
  } else if (o->f32_uniforms) {
    philox_block23(o->seed, c, o->step_ctr, 0u, &uphi, &uth);
  } else {
    philox_block(o->seed, c, o->step_ctr, 0u, &uphi, &uth);
  }
  const double phi = 2. * M_PI * (uphi);
  const double theta = 2. * (uth - 0.5);
  double a[3];
  a[0] = sqrt(1 - theta * theta) * cos(phi);
  a[1] = sqrt(1 - theta * theta) * sin(phi);
  a[2] = theta;
  const double cc = o->rot_c, ss = o->rot_s;
  double R[3][3];
  R[0][0] = a[0] * a[0] + (1 - a[0] * a[0]) * cc;
  R[0][1] = a[0] * a[1] * (1 - cc) - a[2] * ss;
  R[0][2] = a[0] * a[2] * (1 - cc) + a[1] * ss;
  R[1][0] = a[0] * a[1] * (1 - cc) + a[2] * ss;
  R[1][1] = a[1] * a[1] + (1 - a[1] * a[1]) * cc;
  R[1][2] = a[1] * a[2] * (1 - cc) - a[0] * ss;
  R[2][0] = a[0] * a[2] * (1 - cc) - a[1] * ss;
  R[2][1] = a[1] * a[2] * (1 - cc) + a[0] * ss;
  R[2][2] = a[2] * a[2] + (1 - a[2] * a[2]) * cc;
  const int amc = o->p.angular_momentum && (o->c_start[c + 1] - o->c_start[c]) > 2;
  double cmp[3] = {0, 0, 0}, ang[3] = {0, 0, 0};
  if (amc) cell_angular(o, c, cmv, R, cmp, ang);
  for (unsigned k = o->c_start[c]; k < o->c_start[c + 1]; ++k) {
    double* v = pvel(o, o->c_mem[k]);
    double d0 = v[0] - cmv[0], d1 = v[1] - cmv[1], d2 = v[2] - cmv[2];
    double r0 = (R[0][0] * d0 + R[0][1] * d1) + R[0][2] * d2;
    double r1 = (R[1][0] * d0 + R[1][1] * d1) + R[1][2] * d2;
    double r2 = (R[2][0] * d0 + R[2][1] * d1) + R[2][2] * d2;
    v[0] = cmv[0] + r0;
    v[1] = cmv[1] + r1;
    v[2] = cmv[2] + r2;
    if (amc) {
      double x[3];
      ppos(o, o->c_mem[k], x);
      const double q[3] = {x[0] - cmp[0], x[1] - cmp[1], x[2] - cmp[2]};
      v[0] += ang[1] * q[2] - ang[2] * q[1];
      v[1] += ang[2] * q[0] - ang[0] * q[2];
      v[2] += ang[0] * q[1] - ang[1] * q[0];
    }
  }
}

/* MPC::shiftParticles (MPC.cpp:301-311). */
static void shift_particles(smpc_orc* o, const double* s) {
  for (long i = 0; i < o->n_f; ++i) {
    double* x = o->fx + 3 * i;
    x[0] += s[0];
    x[1] += s[1];
    x[2] += s[2];
    wrap_particle(o, x, o->fv + 3 * i);
  }
  for (int m = 0; m < o->n_m; ++m) {
    double* x = o->mx + 3 * m;
    x[0] += s[0];
    x[1] += s[1];
    x[2] += s[2];
  }
}

/* MPC::step (MPC.cpp:116-142). */
void orc_mpc_step(smpc_orc* o, long t, double dt) {
  o->delrx += o->p.shear * o->p.L[1] * (dt * o->p.delrx_dt_scale);
  o->delrx -= o->p.L[0] * round(o->delrx / o->p.L[0]);
  if (t % (long)o->p.step_update) return;
  check_bounds(o);
  for (long i = 0; i < o->n_f; ++i) { /* MPC::streaming (MPC.cpp:192-197) */
    double* x = o->fx + 3 * i;
    const double* v = o->fv + 3 * i;
    x[0] += v[0] * dt;
    x[1] += v[1] * dt;
    x[2] += v[2] * dt;
    wrap_particle(o, x, o->fv + 3 * i);
  }
  double shift[3];
  if (o->rng_mode == ORC_RNG_INJECT) {
    if (!o->inj_shift || !o->inj_uphi || !o->inj_utheta) {
      o->err |= ORC_ERR_INJECT;
      return;
    }
    for (int d = 0; d < 3; ++d) shift[d] = o->inj_shift[d];
  } else {
    double a, b, c;
    philox_block(o->seed, 0xFFFFFFFFu, o->step_ctr, 0u, &a, &b);
    philox_block(o->seed, 0xFFFFFFFFu, o->step_ctr, 1u, &c, NULL);
    shift[0] = a - 0.5;
    shift[1] = b - 0.5;
    shift[2] = c - 0.5;
  }
  shift_particles(o, shift);
  mpc_sort(o);
  const double sLy = o->p.shear * o->p.L[1];
  if (o->p.mono_wrap)
    for (int m = 0; m < o->n_m; ++m) o->mv[3 * m] -= o->m_img[m] * sLy;
  for (unsigned c = 0; c < o->n_cell; ++c) {
    double cmv[3];
    cell_cmv(o, c, cmv);
    cell_thermostat(o, c, cmv);
    cell_collide(o, c, cmv);
  }
  if (o->p.mono_wrap)
    for (int m = 0; m < o->n_m; ++m) o->mv[3 * m] += o->m_img[m] * sLy;
  shift[0] = -shift[0];
  shift[1] = -shift[1];
  shift[2] = -shift[2];
  shift_particles(o, shift);
  if (o->rng_mode == ORC_RNG_PHILOX) o->step_ctr++;
}

void orc_run(smpc_orc* o, long t0, long n, double mpc_dt, int with_md) {
  for (long t = t0; t < t0 + n; ++t) {
    if (with_md) orc_propagate(o, 0);
    orc_mpc_step(o, t, mpc_dt);
  }
}

/* MPC::calculateEkinInCell / EkinTotal / CurrentTemperature / filledCells
 * (MPC.cpp:384-418) on the cell lists of the last collision. */
double orc_temperature(smpc_orc* o) {
  double ekin_tot = 0.0;
  unsigned filled = 0;
  /* monomers binned at a Lees-Edwards image count with that image's velocity,
   * as in the collision (orc_mpc_step) */
  double* vx_saved = NULL;
  if (o->p.mono_wrap && o->n_m > 0) {
    const double sLy = o->p.shear * o->p.L[1];
    vx_saved = (double*)malloc(sizeof(double) * (size_t)o->n_m);
    for (int m = 0; m < o->n_m; ++m) {
      vx_saved[m] = o->mv[3 * m];
      o->mv[3 * m] -= o->m_img[m] * sLy;
    }
  }
  for (unsigned c = 0; c < o->n_cell; ++c) {
    double cmv[3];
    cell_cmv(o, c, cmv);
    double ekin = 0.0;
    unsigned nfl = o->c_fl[c];
    for (unsigned k = 0; k < nfl; ++k) {
      long id = o->c_mem[o->c_start[c] + k];
      const double* v = pvel(o, id);
      double d0 = v[0] - cmv[0], d1 = v[1] - cmv[1], d2 = v[2] - cmv[2];
      ekin += pmass(o, id) * ((d0 * d0 + d1 * d1) + d2 * d2);
    }
    ekin *= 0.5;
    ekin_tot += ekin;
    if (nfl > 0) filled++;
  }
  if (vx_saved) {
    for (int m = 0; m < o->n_m; ++m) o->mv[3 * m] = vx_saved[m];
    free(vx_saved);
  }
  return 2. * ekin_tot / (3. * (unsigned)((unsigned)o->n_f - filled));
}

unsigned orc_n_cells(const smpc_orc* o) { return o->n_cell; }

/* Cell of every solvent particle and monomer in the last collision's cell
 * lists (MPCParticle::CellIndex, MPC.cpp:209,224); -1 for one that was not
 * binned. */
void orc_cell_members(const smpc_orc* o, int* fluid_cell, int* mono_cell) {
  if (fluid_cell)
    for (long i = 0; i < o->n_f; ++i) fluid_cell[i] = -1;
  if (mono_cell)
    for (int m = 0; m < o->n_m; ++m) mono_cell[m] = -1;
  for (unsigned c = 0; c < o->n_cell; ++c)
    for (unsigned k = o->c_start[c]; k < o->c_start[c + 1]; ++k) {
      const long id = o->c_mem[k];
      if (id >= 0) {
        if (fluid_cell) fluid_cell[id] = (int)c;
      } else if (mono_cell) {
        mono_cell[-id - 1] = (int)c;
      }
    }
}

void orc_cell_counts(const smpc_orc* o, unsigned* total, unsigned* fluid) {
  for (unsigned c = 0; c < o->n_cell; ++c) {
    if (total) total[c] = o->c_tot[c];
    if (fluid) fluid[c] = o->c_fl[c];
  }
}

/* ------------------------------------------------------------ periodic MD
 * Many molecules in one periodic Lees-Edwards box. The reference integrates
 * one star without periodic images; this mode restates the GPU's periodic
 * form with the reference's own pieces: Thermostat_None::propagate
 * (Thermostat_None.cpp:21-38), MPC::LEBC for keeping monomers in the primary
 * box (MPC.cpp:421-429), MPC::relative_position for every pair and bond
 * distance (MPC.cpp:456-465) and the potentials of Potentials.h. Pairs are
 * summed over all other monomers in index order (no Verlet list: only pairs
 * inside the potentials' ranges contribute), then each monomer's undirected
 * bonds in bond order, the order the GPU keeps. */

void orc_set_periodic_md(smpc_orc* o, double h) {
  o->periodic = 1;
  o->pmd_h = h;
}

/* delrx one MD step ahead (MPC.cpp:117-118) */
static double pmd_next_delrx(const smpc_orc* o) {
  double d = o->delrx;
  d += o->p.shear * o->p.L[1] * (o->pmd_h * o->p.delrx_dt_scale);
  d -= o->p.L[0] * round(d / o->p.L[0]);
  return d;
}

static inline void pmd_wrap(const smpc_orc* o, double dl, double* x, double* v) {
  const double Lx = o->p.L[0], Ly = o->p.L[1], Lz = o->p.L[2];
  double cy = round(x[1] / Ly);
  x[0] -= Lx * round(x[0] / Lx);
  x[0] -= cy * dl;
  x[0] -= Lx * round(x[0] / Lx);
  x[1] -= Ly * cy;
  x[2] -= Lz * round(x[2] / Lz);
  v[0] -= cy * o->p.shear * Ly;
}

static inline void pmd_min_image(const smpc_orc* o, double dl, double* d) {
  const double Lx = o->p.L[0], Ly = o->p.L[1], Lz = o->p.L[2];
  double cy = round(d[1] / Ly);
  d[0] -= Lx * round(d[0] / Lx);
  d[0] -= cy * dl;
  d[0] -= Lx * round(d[0] / Lx);
  d[1] -= Ly * cy;
  d[2] -= Lz * round(d[2] / Lz);
}

static void pmd_adjacency(smpc_orc* o) {
  const int n = o->n_m;
  free(o->adj_start); free(o->adj_idx); free(o->adj_anchor);
  o->adj_start = (int*)calloc((size_t)n + 2, sizeof(int));
  o->adj_idx = (int*)malloc(sizeof(int) * (size_t)(2 * o->n_bond + 1));
  o->adj_anchor = (unsigned char*)malloc((size_t)(2 * o->n_bond + 1));
  int* fill = (int*)calloc((size_t)n + 1, sizeof(int));
  for (int b = 0; b < o->n_bond; ++b) {
    o->adj_start[o->bsrc[b] + 1]++;
    o->adj_start[o->bdst[b] + 1]++;
  }
  for (int i = 0; i < n; ++i) o->adj_start[i + 1] += o->adj_start[i];
  for (int b = 0; b < o->n_bond; ++b) {
    const int s = o->bsrc[b], d = o->bdst[b];
    int k = o->adj_start[s] + fill[s]++;
    o->adj_idx[k] = d;
    o->adj_anchor[k] = o->anchor[s];
    k = o->adj_start[d] + fill[d]++;
    o->adj_idx[k] = s;
    o->adj_anchor[k] = o->anchor[s];
  }
  free(fill);
}

static int pmd_cell_axis(double x, double L, int nc) {
  int c = (int)floor((x + 0.5 * L) * (nc / L));
  return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

static int cmp_int(const void* a, const void* b) {
  const int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

/* Large boxes: the partners of monomer i come from a periodic grid of cells
 * of side >= r_verlet (the rows beyond a y face looked up at x -/+ delrx),
 * sorted by index, so the sums below see the same non-zero terms in the same
 * order as the loop over all monomers. */
typedef struct {
  int nc[3];
  int* head;
  int* next;
} pmd_grid;

static int pmd_grid_build(const smpc_orc* o, pmd_grid* g) {
  for (int d = 0; d < 3; ++d) {
    g->nc[d] = (int)floor(o->p.L[d] / o->p.r_verlet);
    if (g->nc[d] < 3) return 0;
  }
  const long ncell = (long)g->nc[0] * g->nc[1] * g->nc[2];
  g->head = (int*)malloc(sizeof(int) * (size_t)ncell);
  g->next = (int*)malloc(sizeof(int) * (size_t)(o->n_m + 1));
  for (long c = 0; c < ncell; ++c) g->head[c] = -1;
  for (int i = o->n_m - 1; i >= 0; --i) {
    const double* x = o->mx + 3 * i;
    const long c = pmd_cell_axis(x[0], o->p.L[0], g->nc[0]) +
                   (long)g->nc[0] * (pmd_cell_axis(x[1], o->p.L[1], g->nc[1]) +
                                     (long)g->nc[1] * pmd_cell_axis(x[2], o->p.L[2], g->nc[2]));
    g->next[i] = g->head[c];
    g->head[c] = i;
  }
  return 1;
}

static int pmd_grid_partners(const smpc_orc* o, const pmd_grid* g, double dl, int i, int* out) {
  const double* x = o->mx + 3 * i;
  const int nx = g->nc[0], ny = g->nc[1], nz = g->nc[2];
  const double Lx = o->p.L[0];
  const int cy = pmd_cell_axis(x[1], o->p.L[1], ny), cz = pmd_cell_axis(x[2], o->p.L[2], nz);
  int cnt = 0;
  for (int oz = -1; oz <= 1; ++oz) {
    const int zz = (cz + oz + nz) % nz;
    for (int oy = -1; oy <= 1; ++oy) {
      const int yr = cy + oy, yy = (yr + ny) % ny;
      double xc = x[0];
      if (yr >= ny) xc -= dl;
      if (yr < 0) xc += dl;
      xc -= Lx * round(xc / Lx);
      const int cx = pmd_cell_axis(xc, Lx, nx);
      for (int ox = -1; ox <= 1; ++ox) {
        const long c = (cx + ox + nx) % nx + (long)nx * (yy + (long)ny * zz);
        for (int j = g->head[c]; j >= 0; j = g->next[j])
          if (j != i) out[cnt++] = j;
      }
    }
  }
  qsort(out, (size_t)cnt, sizeof(int), cmp_int);
  return cnt;
}

static void pmd_forces(smpc_orc* o, double dl, int calc_epot) {
  const int n = o->n_m, pot = o->p.potential;
  const double lambda = o->p.lambda;
  for (int m = 0; m < o->n_mol; ++m) o->epot_mol[m] = 0.0;
  pmd_grid grid = {{0, 0, 0}, NULL, NULL};
  const int use_grid = (n > 2048 || o->pmd_force_grid) && pmd_grid_build(o, &grid);
  int* part = (int*)malloc(sizeof(int) * (size_t)(n + 1));
  int mol = 0;
  for (int i = 0; i < n; ++i) {
    while (mol + 1 < o->n_mol && i >= o->mol_start[mol + 1]) ++mol;
    const double* xi = o->mx + 3 * i;
    double F0 = 0.0, F1 = 0.0, F2 = 0.0, ep = 0.0;
    int np = n;
    if (use_grid) np = pmd_grid_partners(o, &grid, dl, i, part);
    for (int q = 0; q < np; ++q) {
      const int j = use_grid ? part[q] : q;
      if (j == i) continue;
      double d[3] = {o->mx[3 * j] - xi[0], o->mx[3 * j + 1] - xi[1], o->mx[3 * j + 2] - xi[2]};
      pmd_min_image(o, dl, d);
      const double r2 = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
      const int bb = (o->amphi[i] == 1 && o->amphi[j] == 1);
      const double fa = pair_force(pot, bb, r2, lambda);
      F0 -= d[0] * fa;
      F1 -= d[1] * fa;
      F2 -= d[2] * fa;
      if (calc_epot) ep += 0.5 * pair_pot(pot, bb, r2, lambda);
    }
    for (int k = o->adj_start[i]; k < o->adj_start[i + 1]; ++k) {
      const int j = o->adj_idx[k];
      const int anch = o->adj_anchor[k];
      double d[3] = {o->mx[3 * j] - xi[0], o->mx[3 * j + 1] - xi[1], o->mx[3 * j + 2] - xi[2]};
      pmd_min_image(o, dl, d);
      double r2 = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
      if (pot != ORC_POT_REF4824) {
        const double cap = (anch ? 20.25 : 2.25) * 0.98;
        if (r2 > cap) r2 = cap;
      }
      const double fa = anch ? fene_anchor_force(r2) : fene_force(r2);
      F0 -= d[0] * fa;
      F1 -= d[1] * fa;
      F2 -= d[2] * fa;
      if (calc_epot) ep += 0.5 * (anch ? fene_anchor_pot(r2) : fene_pot(r2));
    }
    o->mf[3 * i] = F0;
    o->mf[3 * i + 1] = F1;
    o->mf[3 * i + 2] = F2;
    if (o->n_mol > 0) o->epot_mol[mol] += ep;
  }
  free(part);
  free(grid.head);
  free(grid.next);
}

/* Test hook: forces at the current positions by the grid (force_grid = 1) or
 * by the loop over all monomers (0), for checking that both agree. */
void orc_periodic_forces(smpc_orc* o, int force_grid, double* out) {
  const int n = o->n_m;
  double* saved = (double*)malloc(sizeof(double) * (size_t)(3 * n + 3));
  memcpy(saved, o->mf, sizeof(double) * (size_t)(3 * n));
  o->pmd_force_grid = force_grid; /* the size threshold lifted (grids need L >= 3 r_verlet) */
  pmd_forces(o, o->delrx, 0);
  o->pmd_force_grid = 0;
  memcpy(out, o->mf, sizeof(double) * (size_t)(3 * n));
  memcpy(o->mf, saved, sizeof(double) * (size_t)(3 * n));
  free(saved);
}

static void pmd_init(smpc_orc* o) {
  pmd_adjacency(o);
  for (int i = 0; i < o->n_m; ++i) pmd_wrap(o, o->delrx, o->mx + 3 * i, o->mv + 3 * i);
  pmd_forces(o, o->delrx, 0);
}

static void pmd_propagate(smpc_orc* o, int calc_epot) {
  const double dt = o->p.md_dt;
  const double dth = dt * 0.50;
  const double dl = pmd_next_delrx(o);
  for (int i = 0; i < o->n_m; ++i) {
    for (int d = 0; d < 3; ++d) {
      o->mv[3 * i + d] += md_kick(o, o->mf[3 * i + d], o->mm[i], dth);
      o->mx[3 * i + d] += o->mv[3 * i + d] * dt;
    }
    pmd_wrap(o, dl, o->mx + 3 * i, o->mv + 3 * i);
  }
  pmd_forces(o, dl, calc_epot);
  for (int i = 0; i < o->n_m; ++i)
    for (int d = 0; d < 3; ++d) o->mv[3 * i + d] += md_kick(o, o->mf[3 * i + d], o->mm[i], dth);
  if (o->andersen) andersen_step(o);
  o->md_step++;
}
