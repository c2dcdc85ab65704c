"""Benchmark / long-run workloads built on the C ABI.

Named by what they are:
  single_star_50   one star f=10, N_arm=40 (50% solvophobic), 50^3 cells at
                   rho=10 (1.25M solvent), monomer mass 5, shear 0.05
  batched_256      256 independent boxes: f ~ U{3..12}, N_arm ~ U{10..60},
                   solvophobic fraction ~ U[0.2,0.8], L ~ U{16..40}, shear
                   log-uniform in [1e-3, 0.5], seeds 1..256 (system.batched_replica_table)
  single_star_20   one star f=6, N_arm=20, 20^3 cells (80k solvent), the
                   CPU-runnable case
  semidilute_100   64 stars f=8, N_arm=40 (20,544 beads) on a randomised
                   lattice in one periodic 100^3 box (10M solvent), shear 0.1
  large_box_200    16 stars f=12, N_arm=30 (5,776 beads) in one periodic
                   200^3 box (80M solvent), shear 0.05
All use h = 0.1, MD dt = 0.01 (10 substeps per collision), kT = 1, solvent
mass 1 and the 12-6 pair preset (WCA core, LJ attraction to 2.5 between
solvophobic beads) with Verlet skin 0.3. Solvent initial states are drawn on
the device (uniform positions, Maxwell-Boltzmann velocities); stars are
self-avoiding walks from the box centre; in the two star solutions they
interact through the Lees-Edwards minimum image (periodic MD), 50%
solvophobic, and solvent and beads start in the steady linear shear flow.
"""
from __future__ import annotations

import dataclasses
from typing import List, Sequence

import numpy as np

from . import capi, system

H = 0.1
MD_DT = 0.01
N_SUB = 10
R_CUT_LJ = 2.5
SKIN = 0.3
MAX_NB = 256


@dataclasses.dataclass
class Built:
    ctx: capi.Context
    specs: List[system.ReplicaSpec]
    stars: List[system.Star]
    n_fluid: List[int]
    n_mono: List[int]

    @property
    def particles(self) -> int:
        return int(sum(self.n_fluid) + sum(self.n_mono))

    @property
    def n_rep(self) -> int:
        return len(self.specs)

    def close(self):
        self.ctx.close()


def compact_star(spec: system.ReplicaSpec, tries: int = 20) -> system.Star:
    """Self-avoiding-walk star with a mild outward bias; among a few seeded
    attempts the one with the smallest extent (most fit inside the box)."""
    rng = np.random.default_rng(1000 + spec.seed)
    best = None
    for _ in range(tries):
        try:
            st = system.make_star(spec.arms, spec.n_arm, spec.solvophobic_fraction,
                                  spec.mono_mass, spec.kT, rng, bond=0.97, anchor_bond=2.0,
                                  r_min=1.0, outward_bias=0.15)
        except RuntimeError:  # a trapped walk: draw again
            continue
        ext = float(np.abs(st.pos).max())
        if best is None or ext < best[0]:
            best = (ext, st)
        if ext < spec.L / 2 - 1.0:
            break
    return best[1]


def replica_desc(spec: system.ReplicaSpec, star: system.Star) -> dict:
    L = spec.L
    return dict(L=(L, L, L), n_fluid=spec.n_c * L ** 3, n_mono=star.n, mol0_size=star.n,
                kT=spec.kT, shear=spec.shear, h=H, md_dt=MD_DT, seed=spec.seed,
                potential=capi.POT_LJ126, r_cut=R_CUT_LJ, r_verlet=R_CUT_LJ + SKIN,
                **{"lambda": 1.0})


def build(specs: Sequence[system.ReplicaSpec], precision=capi.FP32, rng_mode=capi.RNG_PHILOX,
          mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL, flags=0) -> Built:
    stars = [compact_star(spec) for spec in specs]
    descs = [dict(replica_desc(s, st), flags=flags) for s, st in zip(specs, stars)]
    ctx = capi.Context(descs, precision=precision, rng=rng_mode, mono_bin=mono_bin,
                       delrx_mode=delrx_mode, step_update=N_SUB, max_neighbors=MAX_NB,
                       strict_cells=0)
    for k, (spec, st) in enumerate(zip(specs, stars)):
        ctx.init_solvent(k, seed=spec.seed)
        ctx.set_monomers(k, st.pos, st.vel, np.zeros_like(st.pos), np.full(st.n, st.mass),
                         st.amphi, st.anchor)
        ctx.set_bonds(k, st.bond_src, st.bond_dst)
    ctx.init_md()
    ctx.synchronize()
    return Built(ctx, list(specs), stars, [d["n_fluid"] for d in descs], [st.n for st in stars])


def solution_desc(spec: system.ReplicaSpec, sol: system.StarSolution) -> dict:
    L = spec.L
    return dict(L=(L, L, L), n_fluid=spec.n_c * L ** 3, n_mono=sol.n, mol0_size=sol.stars[0].n,
                kT=spec.kT, shear=spec.shear, h=H, md_dt=MD_DT, seed=spec.seed,
                potential=capi.POT_LJ126, r_cut=R_CUT_LJ, r_verlet=R_CUT_LJ + SKIN,
                flags=capi.REPLICA_PERIODIC_MD, **{"lambda": 1.0})


def make_solution(spec: system.ReplicaSpec) -> system.StarSolution:
    return system.star_solution(spec.n_stars, spec.arms, spec.n_arm, spec.solvophobic_fraction,
                                spec.mono_mass, spec.kT, (spec.L,) * 3,
                                np.random.default_rng(3000 + spec.seed), bond=0.97,
                                outward_bias=0.15)


def build_solution(spec: system.ReplicaSpec, precision=capi.FP32, rng_mode=capi.RNG_PHILOX,
                   delrx_mode=capi.DELRX_PHYSICAL) -> Built:
    """One periodic box holding ``spec.n_stars`` interacting stars."""
    sol = make_solution(spec)
    desc = solution_desc(spec, sol)
    ctx = capi.Context([desc], precision=precision, rng=rng_mode, mono_bin=capi.MONOBIN_WRAPPED,
                       delrx_mode=delrx_mode, step_update=N_SUB, max_neighbors=MAX_NB,
                       strict_cells=0)
    # start in the steady shear flow a long run reaches (v_x += shear * y for
    # solvent and beads), not from rest
    ctx.init_solvent(0, seed=spec.seed, shear_profile=True)
    vel = sol.vel.copy()
    vel[:, 0] += spec.shear * sol.pos[:, 1]
    ctx.set_monomers(0, sol.pos, vel, np.zeros_like(sol.pos), sol.mass, sol.amphi, sol.anchor)
    ctx.set_bonds(0, sol.bond_src, sol.bond_dst)
    ctx.set_molecules(0, sol.mol_start)
    ctx.init_md()
    ctx.synchronize()
    return Built(ctx, [spec], sol.stars, [desc["n_fluid"]], [sol.n])


def semidilute_spec(shear=0.1) -> system.ReplicaSpec:
    return system.ReplicaSpec(L=100, arms=8, n_arm=40, solvophobic_fraction=0.5, shear=shear,
                              seed=1, n_stars=64)


def large_box_spec(shear=0.05) -> system.ReplicaSpec:
    return system.ReplicaSpec(L=200, arms=12, n_arm=30, solvophobic_fraction=0.5, shear=shear,
                              seed=1, n_stars=16)


def semidilute_100(precision=capi.FP32, shear=0.1, **kw) -> Built:
    return build_solution(semidilute_spec(shear), precision=precision, **kw)


def large_box_200(precision=capi.FP32, shear=0.05, **kw) -> Built:
    return build_solution(large_box_spec(shear), precision=precision, **kw)


def single_star_periodic_spec(shear=0.05) -> system.ReplicaSpec:
    return system.ReplicaSpec(L=50, arms=10, n_arm=40, solvophobic_fraction=0.5, shear=shear,
                              seed=1, n_stars=1)


def single_star_50_periodic(precision=capi.FP32, shear=0.05, **kw) -> Built:
    """single_star_50 (the same star, solvent and initial velocities, built by
    ``build``) with its MD through the periodic path: the star's beads spread
    over many CTAs, kept in the primary box and interacting through the
    Lees-Edwards minimum image, with no recentring. That is the reference's
    one-star model (no periodic images, Box.cpp:105-180) as long as no two
    beads of the star are further apart than L - r_cut along an axis, so that
    no bead meets another one's image; ``star_extent`` measures it."""
    spec = system.ReplicaSpec(L=50, arms=10, n_arm=40, solvophobic_fraction=0.5, shear=shear,
                              seed=1)
    return build([spec], precision=precision, flags=capi.REPLICA_PERIODIC_MD, **kw)


def star_extent(built: Built, rep: int = 0) -> np.ndarray:
    """Largest separation along x, y and z between two beads of the replica's
    first molecule after making it whole: every bond (outward from the core,
    bonds in topology order) is placed at its Lees-Edwards minimum image
    (MPC.cpp:456-465) with the current delrx."""
    spec, star = built.specs[rep], built.stars[rep]
    L = float(spec.L)
    pos, _, _ = built.ctx.get_monomers(rep)
    pos = np.array(pos[:star.n], dtype=np.float64)
    delrx = built.ctx.delrx(rep)
    whole = pos.copy()
    for a, b in zip(star.bond_src, star.bond_dst):
        d = pos[b] - whole[a]
        cy = np.round(d[1] / L)
        d[1] -= cy * L
        d[0] -= cy * delrx
        d[0] -= L * np.round(d[0] / L)
        d[2] -= L * np.round(d[2] / L)
        whole[b] = whole[a] + d
    return whole.max(axis=0) - whole.min(axis=0)


SOLUTIONS = ("semidilute_100", "large_box_200")
SOLUTION_SPECS = {"semidilute_100": semidilute_spec, "large_box_200": large_box_spec}
# workloads whose MD runs through the periodic path
PERIODIC = SOLUTIONS + ("single_star_50_periodic",)


def single_star_50(precision=capi.FP32, shear=0.05, **kw) -> Built:
    spec = system.ReplicaSpec(L=50, arms=10, n_arm=40, solvophobic_fraction=0.5, shear=shear,
                              seed=1)
    return build([spec], precision=precision, **kw)


def single_star_20(precision=capi.FP32, shear=0.05, **kw) -> Built:
    spec = system.ReplicaSpec(L=20, arms=6, n_arm=20, solvophobic_fraction=0.5, shear=shear,
                              seed=1)
    return build([spec], precision=precision, **kw)


def batched_256(precision=capi.FP32, n=256, **kw) -> Built:
    """The 256-replica table, or its first n replicas."""
    return build(system.batched_replica_table(256)[:n], precision=precision, **kw)


WORKLOADS = {"batched_256": batched_256, "single_star_50": single_star_50,
             "single_star_20": single_star_20, "semidilute_100": semidilute_100,
             "large_box_200": large_box_200, "single_star_50_periodic": single_star_50_periodic}
