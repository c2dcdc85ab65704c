"""FP32 bulk against the FP64 path on one workload: the precision report of the
large-box stress test (200^3 cells, 80 M solvent particles, 16 stars f = 12,
N_arm = 30, shear 0.05).

Both precisions run the same workload with the same seeds for the same
number of collision cycles. The FP32 and FP64 paths build their uniforms from
different bits of the Philox words, so the two runs are independent samples
of the same ensemble, compared through their averages. Every ``every``
cycles each run reports, with FP64 reductions on the device or on the host:

* total momentum of solvent plus monomers along y and z (x is not conserved
  under Lees-Edwards shear: a particle crossing a y face changes v_x by the
  shear velocity), as drift per particle from the start of the run;
* the temperature against the target kT, twice: the reference's estimator
  (``smpc_temperature_all``, MPC::calculateCurrentTemperature: velocities
  relative to each collision cell's mean, the stored primary-box velocities,
  so a cell straddling a y face counts the Lees-Edwards jump of its
  particles' x velocities) and the kinetic one, sum m u^2 / (3 N) with the
  peculiar velocity u = v - shear y e_x of every particle;
* the xy component of the pressure tensor (kinetic with the peculiar
  velocity, plus the monomer virial), i.e. minus the shear stress;
* the stars' radius-of-gyration tensor (mean over stars).

The report gives, per quantity, the time averages of both runs, their
difference and its standard error from ten block averages of each run, as one
JSON object. In the one-star workloads MPC::check_bounds recentres the world
on the star (MPC.cpp:183-188), subtracting the star's velocity from every
particle; the total momentum then changes with every recentring in both
precisions, so its drift measures precision only in the periodic workloads
(no recentring).

    python -m starpolymersmd_gb300.precision_report --workload large_box_200 \
        --cycles 200 --every 20
    python -m starpolymersmd_gb300.precision_report --workload single_star_50 \
        --shear 0,0.01,0.05,0.2 --cycles 10000 --every 100     # the shear sweep

Each cycle stretch between samples is timed with CUDA events on the
context's stream (ms_per_cycle, sampling excluded).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import capi, workloads as W


def _momentum_yz(ctx, built):
    p = np.zeros(3)
    for k in range(built.n_rep):
        _, fv = ctx.get_fluid(k)
        p += fv.sum(axis=0)  # solvent mass 1
        _, mv, _ = ctx.get_monomers(k)
        p += (mv * built.specs[k].mono_mass).sum(axis=0)
    return p[1:]


def _sample(ctx, built):
    ctx.synchronize()
    kin, vir = ctx.pressure_tensor_all()  # per unit volume
    obs = ctx.molecule_observables_all()
    volume = float(built.specs[0].L) ** 3
    return {
        "p_yz": _momentum_yz(ctx, built),
        "temperature": float(ctx.temperature_all()[0]),
        "temperature_kinetic": float((kin[0, 0] + kin[0, 1] + kin[0, 2]) * volume
                                     / (3.0 * built.particles)),
        "p_xy": float(kin[0, 3] + vir[0, 3]),
        "gyration": obs[0, 1:10].copy(),
    }


def _run(workload, precision, cycles, every, shear=None):
    t0 = time.perf_counter()
    kw = {} if shear is None else {"shear": shear}
    built = W.WORKLOADS[workload](precision=precision, **kw)
    ctx = built.ctx
    n = built.particles
    ctx.synchronize()
    p0 = _momentum_yz(ctx, built)
    samples = []
    cycle_ms = 0.0
    for _ in range(cycles // every):
        cycle_ms += ctx.time_cycles(every)  # CUDA events on the context stream
        samples.append(_sample(ctx, built))
    ctx.raise_on_device_error()
    kT = built.specs[0].kT
    built.close()
    return {
        "momentum_drift_per_particle": [float(np.abs(s["p_yz"] - p0).max() / n) for s in samples],
        "temperature": np.array([s["temperature"] for s in samples]),
        "temperature_kinetic": np.array([s["temperature_kinetic"] for s in samples]),
        "p_xy": np.array([s["p_xy"] for s in samples]),
        "gyration": np.array([s["gyration"] for s in samples]),
        "kT": kT,
        "seconds": time.perf_counter() - t0,
        "ms_per_cycle": cycle_ms / max(1, (cycles // every) * every),
    }


N_BLOCKS = 10


def _mean_err(x):
    """Mean and its standard error from N_BLOCKS block means: samples a few
    hundred collisions apart are still correlated (a star's shape relaxes
    slowly), so the spread of single samples would understate the error."""
    x = np.asarray(x, dtype=np.float64)
    m = x.mean(axis=0)
    nb = min(N_BLOCKS, len(x))
    if nb < 2:
        return m, np.zeros_like(m)
    per = len(x) // nb
    blocks = x[: per * nb].reshape((nb, per) + x.shape[1:]).mean(axis=1)
    return m, blocks.std(axis=0, ddof=1) / np.sqrt(nb)


def report(workload="large_box_200", cycles=200, every=20, shear=None):
    runs = {name: _run(workload, prec, cycles, every, shear)
            for name, prec in (("fp32", capi.FP32), ("fp64", capi.FP64))}
    out = {"workload": workload, "cycles": cycles, "sample_every": every,
           "seconds": {k: round(v["seconds"], 1) for k, v in runs.items()},
           "ms_per_cycle": {k: round(v["ms_per_cycle"], 4) for k, v in runs.items()}}
    if shear is not None:
        out["shear"] = shear
    for key in ("temperature", "temperature_kinetic", "p_xy", "gyration"):
        m32, e32 = _mean_err(runs["fp32"][key])
        m64, e64 = _mean_err(runs["fp64"][key])
        out[key] = {"fp32": np.round(m32, 6).tolist(), "fp64": np.round(m64, 6).tolist(),
                    "fp32_minus_fp64": np.round(m32 - m64, 6).tolist(),
                    "std_error_of_difference": np.round(np.sqrt(e32 ** 2 + e64 ** 2), 6).tolist()}
    for key in ("temperature", "temperature_kinetic"):
        out[key]["target_kT"] = runs["fp32"]["kT"]
        for name in ("fp32", "fp64"):
            out[key][name + "_error_vs_kT"] = round(float(np.mean(runs[name][key])
                                                          - runs[name]["kT"]), 6)
    out["momentum_yz_drift_per_particle"] = {
        k: float(max(v["momentum_drift_per_particle"])) for k, v in runs.items()}
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="large_box_200", choices=sorted(W.WORKLOADS))
    ap.add_argument("--cycles", type=int, default=200)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--shear", default=None,
                    help="comma-separated shear rates: one report per rate (a sweep)")
    a = ap.parse_args()
    if a.shear is None:
        print(json.dumps(report(a.workload, a.cycles, a.every)), flush=True)
    else:
        for g in (float(x) for x in a.shear.split(",")):
            print(json.dumps(report(a.workload, a.cycles, a.every, g)), flush=True)


if __name__ == "__main__":
    main()
