"""Long runs of the GPU paths against the reference's own long run.

tests/golden/longrun_config1.npz holds block averages of a run of the
reference compiled from its own sources (tests/golden/make_longrun.py): the
first benchmark configuration's star (f = 6, A = B = 10, mass 5, 48-24
potentials) and solvent (N_c = 10, kT = 1, shear 0.05, h = 0.1, 10 MD
substeps) in a 50^3 box, 1000 + 10,000 collisions, sampled every 10. The FP64
and the FP32 GPU path run the same system from the same initial state with
their own (Philox) random numbers for the same number of collisions, and each
average must agree with the reference's within statistical error: the
difference below 4 combined standard errors of the block means. Compared:
  * the temperature estimator MPC::calculateCurrentTemperature (MPC.cpp:405-409),
  * the gyration tensor G_xx, G_xy, G_yy, G_zz and R_g (Box.cpp:330-353),
  * the rotation frequency about z (Box.cpp:355-379),
  * the polymer temperature (Box.cpp:635-646),
  * the slope of the VelocityX profile v_x(y) (Velocity_x.h:76-100), which
    must also equal the shear rate within 4 standard errors (the linear
    profile the reference's results/plot_MPC_tests.py:59-60 compares with).
"""
import os

import numpy as np
import pytest

from starpolymersmd_gb300 import capi
from tests.golden import make_longrun as M

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "longrun_config1.npz")

# sample-row columns (make_longrun.sample_row): T_est, then the 16 observables
COLS = {"T_est": 0, "R_g": 1, "G_xx": 2, "G_xy": 3, "G_yy": 6, "G_zz": 10, "omega_z": 13,
        "T_polymer": 15}
OBS0 = 1
PROF0 = 17


def profile_slopes(blocks, L, width):
    """Least-squares slope of the mean v_x per y bin against the bin centre,
    per block (bins with particles only)."""
    nb = (blocks.shape[1] - PROF0) // 3
    k0 = np.floor(-L / (2.0 * width))
    yc = (np.arange(nb) + k0 + 0.5) * width
    out = []
    for b in blocks:
        prof = b[PROF0:].reshape(nb, 3)
        ok = prof[:, 2] > 0
        vx = prof[ok, 0] / prof[ok, 2]
        y = yc[ok]
        out.append(((y - y.mean()) * (vx - vx.mean())).sum() / ((y - y.mean()) ** 2).sum())
    return np.array(out)


def mean_se(x):
    x = np.asarray(x)
    return float(x.mean()), float(x.std(ddof=1) / np.sqrt(len(x)))


def run_gpu(fx, precision):
    L = int(fx["L"])
    pos, vel = M.initial_fluid()
    n_m = len(fx["star_pos"])
    rep = dict(L=(L,) * 3, n_fluid=len(pos), n_mono=n_m, mol0_size=n_m, kT=float(fx["kT"]),
               shear=float(fx["shear"]), h=float(fx["h"]), md_dt=float(fx["md_dt"]),
               seed=2024 + precision, **{"lambda": float(fx["lam"])})
    rows = []
    with capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX,
                      step_update=int(fx["n_sub"]), mono_bin=capi.MONOBIN_REFERENCE,
                      delrx_mode=capi.DELRX_PHYSICAL,
                      strict_cells=1 if precision == capi.FP64 else 0) as ctx:
        ctx.set_fluid(0, pos, vel)
        ctx.set_monomers(0, fx["star_pos"], fx["star_vel"], np.zeros_like(fx["star_pos"]),
                         fx["star_mass"], fx["star_amphi"], fx["star_anchor"])
        ctx.set_bonds(0, fx["bond_src"], fx["bond_dst"])
        ctx.init_md()
        ctx.cycles(int(fx["equil"]))
        every = int(fx["sample"])
        for _ in range(int(fx["prod"]) // every):
            ctx.cycles(every)
            T = ctx.temperature(0)
            obs = ctx.molecule_observables_all()[0]
            _, py = ctx.velocity_profile(0, float(fx["width"]))
            rows.append(M.sample_row(T, obs, py))
        ctx.raise_on_device_error()
    rows = np.array(rows)
    nb = fx["blocks"].shape[0]
    per = len(rows) // nb
    return rows[: per * nb].reshape(nb, per, -1).mean(axis=1)


@pytest.fixture(scope="module")
def fx():
    if not os.path.exists(FIXTURE):
        pytest.skip("long-run fixture not generated")
    return dict(np.load(FIXTURE))


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32], ids=["fp64", "fp32"])
def test_long_run_agrees_with_reference(fx, precision, record_property):
    ref = fx["blocks"]
    gpu = run_gpu(fx, precision)
    assert gpu.shape == ref.shape
    report = {}
    for name, c in COLS.items():
        mg, sg = mean_se(gpu[:, c])
        mr, sr = mean_se(ref[:, c])
        report[name] = (mg, mr, sg, sr)
        assert abs(mg - mr) < 4.0 * np.hypot(sg, sr), (name, report[name])
    L, w = int(fx["L"]), float(fx["width"])
    sg_, sr_ = profile_slopes(gpu, L, w), profile_slopes(ref, L, w)
    mg, sg = mean_se(sg_)
    mr, sr = mean_se(sr_)
    assert abs(mg - mr) < 4.0 * np.hypot(sg, sr), ("slope", mg, mr, sg, sr)
    report["slope"] = (mg, mr, sg, sr)
    record_property("gpu_ref_segse", report)
    shear = float(fx["shear"])
    assert abs(mg - shear) < 4.0 * sg + 0.02 * shear, ("slope vs shear", mg, sg)
    assert abs(mr - shear) < 4.0 * sr + 0.02 * shear, ("reference slope vs shear", mr, sr)
