"""Long-run statistics of config 1 from the reference compiled from its own
sources (oracle/refbuild): the fixture tests/golden/longrun/longrun_config1.npz that
tests/test_gpu_longrun.py compares the GPU paths with.

System: the first benchmark configuration's star and solvent -- one star of
f = 6 arms with A = B = 10 monomers (121 beads, mass 5; the outer half of
every arm solvophobic, the reference's 48-24 potentials with lambda = 1),
MPC cells at N_c = 10, kT = 1, shear rate 0.05, rotation angle 130 degrees,
collision step h = 0.1, MD step 0.01 (10 velocity-Verlet substeps per
collision) -- in a 50^3 box (1.25 M solvent particles, the second
configuration's box). The configuration's 20^3 box is too small for the
reference's model over a long run: its Verlet grid is bounded by the box
around the star's centre (Box.cpp:105-142), and in the shear flow an arm is
drawn out along x towards its contour length of about 21 (extent from the
centre 9.5 -> 16.8 over the first 580 collisions in a 30^3 box), past the half
width of 10 (or 15) within a few hundred collisions, where the reference
raises SIGSEGV.

Driving: the library-level loop of gaussian_chain.cpp:347-352 and
star-polymers.cpp:530-534 with step_update = 1 and MPC::step(t, h) called once
after every 10 Thermostat_None::propagate calls, so delrx advances by
shear * L_y * h per collision (the physical Lees-Edwards offset; calling it
every MD step with step_update = 10 advances it ten times too fast,
MPC.cpp:117-119). The star has the reference's layout and bonds
(Box::add_star) but starts as a compact self-avoiding walk from the box centre
(system.make_star, seed 1; the reference's straight-ray arms of 20 beads
start at the grid's edge), written in with ref_set_monomers; the solvent starts
uniform in the box with Maxwell-Boltzmann velocities at kT plus the steady
flow shear * y, mean removed. Both come from numpy's PCG64 and are regenerated
by the test with the same calls.

Recorded: RUNS independent trajectories from the same initial star (solvent
from numpy seed FLUID_SEED + k, the reference's random stream re-seeded with
RAND_SEED + k), run in parallel processes. For each, after EQUIL cycles,
every SAMPLE-th of PROD cycles:
  T_est   MPC::calculateCurrentTemperature (MPC.cpp:405-409),
  obs     Box observables after center_of_mass_reference_frame (R_g, gyration
          tensor, rotation frequency, kinetic energy, polymer temperature;
          Box.cpp:288-379, 635-646),
  prof_y  VelocityX along y with bins of width 1 (Velocity_x.h:76-100),
kept as the means over BLOCKS consecutive blocks of each run. A stretched
star tumbling in shear flow decorrelates slowly, so the comparison uses the
spread of the run means, not blocks of one run.

    SMPC_REFERENCE=<reference checkout> python tests/golden/make_longrun.py
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from starpolymersmd_gb300 import system  # noqa: E402

L, NC, KT, SHEAR, MASS, LAM = 50, 10, 1.0, 0.05, 5.0, 1.0
ARMS, A, B = 6, 10, 10
H_MPC, MD_DT, N_SUB = 0.1, 0.01, 10
EQUIL, PROD, SAMPLE, BLOCKS = 1000, 10000, 10, 10
RUNS = 8
WIDTH = 1.0
FLUID_SEED = 1
STAR_SEED = 1
RAND_SEED = 1000


def initial_star():
    """Compact self-avoiding star (reference layout: core 0, arm i bead k at
    i (A + B) + k) within 8.5 of the centre."""
    rng = np.random.default_rng(STAR_SEED)
    for _ in range(200):
        star = system.make_star(ARMS, A + B, B / (A + B), MASS, KT, rng, bond=1.01,
                                outward_bias=0.0)
        if np.abs(star.pos).max() < 8.5:
            return star
    raise RuntimeError("no compact star")


def initial_fluid(run=0):
    """Uniform positions, Maxwell-Boltzmann velocities at KT, mean removed,
    plus the steady linear flow SHEAR * y along x."""
    rng = np.random.default_rng(FLUID_SEED + run)
    n = NC * L ** 3
    pos = (rng.random((n, 3)) - 0.5) * L
    vel = rng.normal(0.0, np.sqrt(KT), (n, 3))
    vel -= vel.mean(axis=0)
    vel[:, 0] += SHEAR * pos[:, 1]
    return pos, vel


def sample_row(T, obs, prof_y):
    return np.concatenate([[T], obs, prof_y.ravel()])


def one_run(run):
    """Block means (BLOCKS x columns) of one trajectory of the reference."""
    ref = orc.RefSystem((L, L, L), KT, LAM, NC, SHEAR, 1)
    ref.reseed(RAND_SEED + run)
    ref.add_star(A, B, ARMS, MASS)
    star = initial_star()
    ref.set_monomers(star.pos, star.vel)
    ref.make_thermostat(MD_DT)
    pos, vel = initial_fluid(run)
    ref.set_fluid(pos, vel)
    rows = []
    t = 0
    for c in range(EQUIL + PROD):
        for _ in range(N_SUB):
            ref.propagate(False)
        ref.mpc_step(t, H_MPC)
        t += 1
        if c >= EQUIL and (c - EQUIL + 1) % SAMPLE == 0:
            T = ref.temperature()
            obs = ref.observables()
            _, py = ref.velocity_profile(WIDTH)
            rows.append(sample_row(T, obs, py))
    rows = np.array(rows)
    per = len(rows) // BLOCKS
    return rows[: per * BLOCKS].reshape(BLOCKS, per, -1).mean(axis=1)


def main():
    ref = orc.RefSystem((L, L, L), KT, LAM, NC, SHEAR, 1)
    ref.add_star(A, B, ARMS, MASS)
    star = initial_star()
    ref.set_monomers(star.pos, star.vel)
    star0 = ref.get_monomers()
    bsrc, bdst = ref.bonds()
    assert np.array_equal(star0["amphi"], star.amphi) and np.array_equal(star0["anchor"], star.anchor)
    del ref
    t0 = time.time()
    with mp.get_context("spawn").Pool(min(RUNS, os.cpu_count() or 1)) as pool:
        blocks = np.array(pool.map(one_run, range(RUNS)))
    out = os.path.join(HERE, "longrun", "longrun_config1.npz")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    np.savez_compressed(
        out, blocks=blocks, L=L, n_c=NC, kT=KT, shear=SHEAR, mass=MASS, lam=LAM, arms=ARMS,
        A=A, B=B, h=H_MPC, md_dt=MD_DT, n_sub=N_SUB, equil=EQUIL, prod=PROD, sample=SAMPLE,
        width=WIDTH, fluid_seed=FLUID_SEED, star_seed=STAR_SEED, rand_seed=RAND_SEED,
        star_pos=star0["pos"], star_vel=star0["vel"], star_mass=star0["mass"],
        star_amphi=star0["amphi"], star_anchor=star0["anchor"], bond_src=bsrc, bond_dst=bdst,
        columns=np.array(["T_est"] + [f"obs{k}" for k in range(16)] +
                         [f"prof{k}_{q}" for k in range(orc.profile_bins(L, WIDTH))
                          for q in ("vx", "vy", "n")]))
    runs = blocks.mean(axis=1)
    m = runs.mean(axis=0)
    se = runs.std(axis=0, ddof=1) / np.sqrt(RUNS)
    print(f"{RUNS} runs in {time.time() - t0:.0f} s -> {out}")
    print(f"T_est {m[0]:.5f} +- {se[0]:.5f}; R_g {m[1]:.4f} +- {se[1]:.4f}; "
          f"polymer T {m[15]:.4f} +- {se[15]:.4f}")


if __name__ == "__main__":
    main()
