"""Long runs of the GPU paths against the reference's own long runs.

tests/golden/longrun/longrun_config1.npz holds block averages of 8
independent runs of the reference compiled from its own sources
(tests/golden/make_longrun.py): the first benchmark configuration's star
(f = 6, A = B = 10, mass 5, 48-24 potentials) and solvent (N_c = 10, kT = 1,
shear 0.05, h = 0.1, 10 MD substeps) in a 50^3 box, 1000 + 10,000 collisions
each, sampled every 10. The FP64 and the FP32 GPU path run 8 trajectories of
the same system from the same initial states (one batched context, each
replica with its own Philox stream) for the same number of collisions.

A stretched star tumbling in shear flow decorrelates slowly, so every
quantity is compared through the means of the runs: the GPU average and the
reference's must differ by less than 5 standard errors of the difference,
each estimated from the spread of its 8 runs (a t distribution with about 14
degrees of freedom: a false alarm about once in 500 runs of this test over
its nine quantities). Compared:
  * the temperature estimator MPC::calculateCurrentTemperature (MPC.cpp:405-409),
  * the gyration tensor G_xx, G_xy, G_yy, G_zz and R_g (Box.cpp:330-353),
  * the rotation frequency about z (Box.cpp:355-379),
  * the polymer temperature (Box.cpp:635-646),
  * the slope of the VelocityX profile v_x(y) (Velocity_x.h:76-100), which
    must also equal the shear rate to 2 % (the linear profile the reference's
    results/plot_MPC_tests.py:59-60 compares with).
"""
import os

import numpy as np
import pytest

from starpolymersmd_gb300 import capi
from tests.golden import make_longrun as M

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "longrun", "longrun_config1.npz")

# sample-row columns (make_longrun.sample_row): T_est, then the 16 observables
COLS = {"T_est": 0, "R_g": 1, "G_xx": 2, "G_xy": 3, "G_yy": 6, "G_zz": 10, "omega_z": 13,
        "T_polymer": 15}
PROF0 = 17
N_SIGMA = 5.0


def profile_slope(row, L, width):
    """Least-squares slope of the mean v_x per y bin against the bin centre
    (bins with particles only) of one run's averaged sample row."""
    nb = (len(row) - PROF0) // 3
    k0 = np.floor(-L / (2.0 * width))
    yc = (np.arange(nb) + k0 + 0.5) * width
    prof = row[PROF0:].reshape(nb, 3)
    ok = prof[:, 2] > 0
    vx = prof[ok, 0] / prof[ok, 2]
    y = yc[ok]
    return ((y - y.mean()) * (vx - vx.mean())).sum() / ((y - y.mean()) ** 2).sum()


def mean_se(x):
    x = np.asarray(x)
    return float(x.mean()), float(x.std(ddof=1) / np.sqrt(len(x)))


def run_gpu(fx, precision):
    """Block means (runs x blocks x columns) of the GPU runs."""
    L = int(fx["L"])
    n_runs, n_blocks = fx["blocks"].shape[:2]
    n_m = len(fx["star_pos"])
    fluids = [M.initial_fluid(k) for k in range(n_runs)]
    reps = [dict(L=(L,) * 3, n_fluid=len(fluids[k][0]), n_mono=n_m, mol0_size=n_m,
                 kT=float(fx["kT"]), shear=float(fx["shear"]), h=float(fx["h"]),
                 md_dt=float(fx["md_dt"]), seed=2024 + 100 * precision + k,
                 **{"lambda": float(fx["lam"])}) for k in range(n_runs)]
    rows = [[] for _ in range(n_runs)]
    with capi.Context(reps, precision=precision, rng=capi.RNG_PHILOX,
                      step_update=int(fx["n_sub"]), mono_bin=capi.MONOBIN_REFERENCE,
                      delrx_mode=capi.DELRX_PHYSICAL,
                      strict_cells=1 if precision == capi.FP64 else 0) as ctx:
        for k, (pos, vel) in enumerate(fluids):
            ctx.set_fluid(k, pos, vel)
            ctx.set_monomers(k, fx["star_pos"], fx["star_vel"], np.zeros_like(fx["star_pos"]),
                             fx["star_mass"], fx["star_amphi"], fx["star_anchor"])
            ctx.set_bonds(k, fx["bond_src"], fx["bond_dst"])
        ctx.init_md()
        ctx.cycles(int(fx["equil"]))
        every = int(fx["sample"])
        for _ in range(int(fx["prod"]) // every):
            ctx.cycles(every)
            temps = ctx.temperature_all()
            obs = ctx.molecule_observables_all()
            for k in range(n_runs):
                _, py = ctx.velocity_profile(k, float(fx["width"]))
                rows[k].append(M.sample_row(temps[k], obs[k], py))
        ctx.raise_on_device_error()
    rows = np.array(rows)
    per = rows.shape[1] // n_blocks
    return rows[:, : per * n_blocks].reshape(n_runs, n_blocks, per, -1).mean(axis=2)


@pytest.fixture(scope="module")
def fx():
    if not os.path.exists(FIXTURE):
        pytest.skip("long-run fixture not generated")
    return dict(np.load(FIXTURE))


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32], ids=["fp64", "fp32"])
def test_long_run_agrees_with_reference(fx, precision, record_property):
    ref = fx["blocks"].mean(axis=1)  # runs x columns
    gpu_blocks = run_gpu(fx, precision)
    assert gpu_blocks.shape == fx["blocks"].shape
    gpu = gpu_blocks.mean(axis=1)
    report = {}
    L, w = int(fx["L"]), float(fx["width"])
    quantities = {name: (gpu[:, c], ref[:, c]) for name, c in COLS.items()}
    quantities["slope"] = (np.array([profile_slope(r, L, w) for r in gpu]),
                           np.array([profile_slope(r, L, w) for r in ref]))
    for name, (g, r) in quantities.items():
        mg, sg = mean_se(g)
        mr, sr = mean_se(r)
        report[name] = (mg, mr, sg, sr)
    record_property("gpu_ref_mean_se", report)
    for name, (mg, mr, sg, sr) in report.items():
        assert abs(mg - mr) < N_SIGMA * np.hypot(sg, sr), (name, report[name])
    shear = float(fx["shear"])
    for who, k in (("gpu", 0), ("reference", 1)):
        assert abs(report["slope"][k] - shear) < 0.02 * shear, (who, report["slope"])
