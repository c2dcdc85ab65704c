"""Statistics of the reference's Lowe-Andersen thermostat (MPC off) from the
reference compiled from its own sources (oracle/refbuild, where the one member
the reference declares without defining is supplied): the fixture
tests/golden/lowe/lowe_star.npz that tests/test_gpu_thermostat.py compares the
GPU's Lowe-Andersen with.

System: one star of f = 6 arms with A = B = 5 monomers (61 beads, mass 5,
48-24 potentials with lambda = 1) alone in a 30^3 box, velocity Verlet with
dt = 0.01 and Lowe_Andersen{box, dt, T = 1, nu = 20, r = 1.5} (the parameters
star-polymers.cpp:388 and gaussian_chain.cpp:382 construct it with). The star
starts as a compact self-avoiding walk (numpy seed STAR_SEED) with
Maxwell-Boltzmann velocities at T of zero total momentum, written into the
reference's star (Box::add_star layout) with ref_set_monomers.

Recorded for RUNS independent runs (the reference's random stream re-seeded
with RAND_SEED + k), after EQUIL steps, over STEPS steps sampled every step:
  t_kin     sum m v^2 / (3 (N - 1)) (the total momentum is conserved at zero),
  p_drift   the largest change of the total momentum over the run,
  vacf      <v_i(t) . v_i(t + tau)> / <v_i . v_i> over beads and time origins at
            the lags LAGS (steps).

    SMPC_REFERENCE=<reference checkout> python tests/golden/make_lowe.py
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

L, KT, MASS, LAM = 30, 1.0, 5.0, 1.0
ARMS, A, B = 6, 5, 5
DT, NU, RADIUS = 0.01, 20.0, 1.5
EQUIL, STEPS, RUNS = 2000, 40000, 8
LAGS = (1, 2, 5, 10, 20, 50)
STAR_SEED, RAND_SEED = 3, 500


def initial_star():
    rng = np.random.default_rng(STAR_SEED)
    star = system.make_star(ARMS, A + B, B / (A + B), MASS, KT, rng, bond=1.01, outward_bias=0.0)
    star.vel -= star.vel.mean(axis=0)
    return star


class VacfAccumulator:
    """<v_i(t) . v_i(t + lag)> over beads and time origins for lags 0..max."""

    def __init__(self, max_lag):
        self.max_lag = max_lag
        self.ring = []
        self.sums = np.zeros(max_lag + 1)
        self.counts = np.zeros(max_lag + 1)

    def push(self, v):
        self.ring.append(np.array(v))
        if len(self.ring) > self.max_lag + 1:
            self.ring.pop(0)
        cur = self.ring[-1]
        for lag in range(len(self.ring)):
            self.sums[lag] += float((self.ring[-1 - lag] * cur).sum())
            self.counts[lag] += 1

    def normalised(self, lags):
        c = self.sums / self.counts
        return np.array([c[l] / c[0] for l in lags])


def statistics(vel_samples, mass):
    """(t_kin, p_drift, vacf at LAGS) of one run's velocity samples."""
    n = vel_samples[0].shape[0]
    acc = VacfAccumulator(max(LAGS))
    t_sum, p0, drift = 0.0, None, 0.0
    for v in vel_samples:
        t_sum += float((mass[:, None] * v * v).sum()) / (3.0 * (n - 1))
        p = (mass[:, None] * v).sum(axis=0)
        if p0 is None:
            p0 = p
        drift = max(drift, float(np.abs(p - p0).max()))
        acc.push(v)
    return t_sum / len(vel_samples), drift, acc.normalised(LAGS)


def one_run(run):
    ref = orc.RefSystem((L, L, L), KT, LAM, 1, 0.0, 1)
    ref.reseed(RAND_SEED + run)
    ref.add_star(A, B, ARMS, MASS)
    star = initial_star()
    ref.set_monomers(star.pos, star.vel)
    ref.make_lowe_andersen(DT, KT, NU, RADIUS)
    for _ in range(EQUIL):
        ref.propagate(False)
    samples = []
    for _ in range(STEPS):
        ref.propagate(False)
        samples.append(ref.get_monomers()["vel"])
    mass = ref.get_monomers()["mass"]
    t_kin, drift, vacf = statistics(samples, mass)
    return np.concatenate([[t_kin, drift], vacf])


def main():
    ref = orc.RefSystem((L, L, L), KT, LAM, 1, 0.0, 1)
    ref.add_star(A, B, ARMS, MASS)
    star = initial_star()
    ref.set_monomers(star.pos, star.vel)
    m0 = ref.get_monomers()
    bsrc, bdst = ref.bonds()
    del ref
    t0 = time.time()
    with mp.get_context("spawn").Pool(min(RUNS, os.cpu_count() or 1)) as pool:
        runs = np.array(pool.map(one_run, range(RUNS)))
    out = os.path.join(HERE, "lowe", "lowe_star.npz")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    np.savez_compressed(out, runs=runs, lags=np.array(LAGS), L=L, kT=KT, mass=MASS, lam=LAM,
                        dt=DT, nu=NU, radius=RADIUS, equil=EQUIL, steps=STEPS,
                        star_pos=m0["pos"], star_vel=m0["vel"], star_mass=m0["mass"],
                        star_amphi=m0["amphi"], star_anchor=m0["anchor"], bond_src=bsrc,
                        bond_dst=bdst)
    m = runs.mean(axis=0)
    se = runs.std(axis=0, ddof=1) / np.sqrt(RUNS)
    print(f"{RUNS} runs in {time.time() - t0:.0f} s -> {out}")
    print("t_kin %.4f +- %.4f, max momentum drift %.2e" % (m[0], se[0], runs[:, 1].max()))
    print("vacf", " ".join(f"{a:.4f}+-{b:.4f}" for a, b in zip(m[2:], se[2:])))


if __name__ == "__main__":
    main()
