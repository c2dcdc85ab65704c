"""Andersen stochastic thermostat of MPC-off runs (SMPC_MDTHERMO_ANDERSEN)
against the oracle's restatement of AndersenStochastic::propagate
(Andersen_stochastic.cpp:30-59) on the same Philox draws, for one star and
for a periodic many-star box, and its temperature on a long FP32 run."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from starpolymersmd_gb300 import capi, system
from tests import gpu_helpers as H
from tests.test_gpu_periodic import _solution

pytestmark = pytest.mark.gpu

NU, SEED = 5.0, 41


def test_fp64_andersen_one_star_matches_oracle():
    L = 12
    star, fpos, fvel = H.small_star_system(L=L, seed=6)
    fpos = fvel = np.zeros((0, 3))
    n = star.n
    o = orc.OracleSystem((L, L, L), 1.0, 0.0, 1000, 0, n, mol_start=[0, n])
    o.set_monomers(star.pos, star.vel, np.zeros_like(star.pos), np.full(n, star.mass),
                   star.amphi, star.anchor)
    o.set_bonds(star.bond_src, star.bond_dst)
    o.set_andersen(NU, SEED)
    o.init_md()
    rep = dict(L=(L, L, L), n_fluid=0, n_mono=n, mol0_size=n, kT=1.0, shear=0.0, h=0.1,
               md_dt=0.01, seed=SEED, **{"lambda": 1.0})
    with capi.Context([rep], precision=capi.FP64, rng=capi.RNG_PHILOX, step_update=1000,
                      md_thermostat=capi.MDTHERMO_ANDERSEN, andersen_nu=NU) as ctx:
        ctx.set_monomers(0, star.pos, star.vel, np.zeros_like(star.pos), np.full(n, star.mass),
                         star.amphi, star.anchor)
        ctx.set_bonds(0, star.bond_src, star.bond_dst)
        ctx.init_md()
        before = ctx.get_monomers(0)[1].copy()
        for _ in range(40):
            o.propagate(False)
        ctx.md_substeps(25)
        ctx.md_substeps(15)  # the draws follow the MD step counter across calls
        ctx.raise_on_device_error()
        mp, mv, mf = ctx.get_monomers(0)
        op, ov, of = o.get_monomers()
        H.close64(mp, op, rtol=1e-11)
        H.close64(mv, ov, rtol=1e-11)
        H.close64(mf, of, rtol=1e-11)
        # with nu dt = 0.05 most beads were redrawn at least once
        assert np.mean(np.any(mv != before, axis=1)) > 0.5


def test_fp64_andersen_periodic_box_matches_oracle():
    L = 12
    sol = _solution(seed=8)
    fpos = np.zeros((0, 3))
    su, md_dt = 1000, 0.005
    o = orc.OracleSystem((L, L, L), 1.0, 0.3, su, 0, sol.n, mol_start=sol.mol_start, md_dt=md_dt,
                         r_verlet=1.8, delrx_dt_scale=1.0 / su, mono_wrap=1)
    o.set_monomers(sol.pos, sol.vel, np.zeros_like(sol.pos), sol.mass, sol.amphi, sol.anchor)
    o.set_bonds(sol.bond_src, sol.bond_dst)
    o.set_periodic_md(su * md_dt)
    o.set_andersen(NU, SEED)
    o.init_md()
    rep = dict(L=(L, L, L), n_fluid=0, n_mono=sol.n, mol0_size=sol.stars[0].n, kT=1.0,
               shear=0.3, h=su * md_dt, md_dt=md_dt, seed=SEED, r_verlet=1.8,
               flags=capi.REPLICA_PERIODIC_MD, **{"lambda": 1.0})
    with capi.Context([rep], precision=capi.FP64, rng=capi.RNG_PHILOX, step_update=su,
                      mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL,
                      md_thermostat=capi.MDTHERMO_ANDERSEN, andersen_nu=NU) as ctx:
        ctx.set_monomers(0, sol.pos, sol.vel, np.zeros_like(sol.pos), sol.mass, sol.amphi,
                         sol.anchor)
        ctx.set_bonds(0, sol.bond_src, sol.bond_dst)
        ctx.init_md()
        for t in range(1, 61):
            o.propagate(False)
            o.mpc_step(t, su * md_dt)  # delrx advance only
        ctx.md_substeps(60)
        ctx.raise_on_device_error()
        for x, y in zip(ctx.get_monomers(0), o.get_monomers()):
            H.close64(x, y, rtol=1e-11)


def test_fp32_andersen_holds_the_temperature():
    L, kT = 16, 1.5
    sol = system.star_solution(6, 4, 8, 0.5, 5.0, 0.2, (L, L, L), np.random.default_rng(12))
    rep = dict(L=(L, L, L), n_fluid=0, n_mono=sol.n, mol0_size=sol.stars[0].n, kT=kT, shear=0.0,
               h=10.0, md_dt=0.01, seed=SEED, potential=capi.POT_LJ126, r_cut=2.5,
               r_verlet=2.8, flags=capi.REPLICA_PERIODIC_MD, **{"lambda": 1.0})
    with capi.Context([rep], precision=capi.FP32, rng=capi.RNG_PHILOX, step_update=1000,
                      mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL,
                      strict_cells=0, md_thermostat=capi.MDTHERMO_ANDERSEN,
                      andersen_nu=2.0) as ctx:
        ctx.set_monomers(0, sol.pos, sol.vel, np.zeros_like(sol.pos), sol.mass, sol.amphi,
                         sol.anchor)
        ctx.set_bonds(0, sol.bond_src, sol.bond_dst)
        ctx.init_md()
        ctx.md_substeps(1000)
        temps = []
        for _ in range(20):
            ctx.md_substeps(50)
            _, v, _ = ctx.get_monomers(0)
            temps.append((sol.mass[:, None] * v * v).sum() / (3 * sol.n))
        ctx.raise_on_device_error()
        assert abs(np.mean(temps) / kT - 1.0) < 0.05


def test_staged_resets_over_several_substeps_and_replicas(golden_dir):
    # the reference fixture's resets staged four substeps at a time into
    # replica 0, while replica 1 (same star) draws from Philox like the oracle
    import os
    from tests import golden_replay as gr
    fx = gr.load(os.path.join(golden_dir, "andersen_m1_L12.npz"))
    n = len(fx["mono_pos0"])
    L = tuple(int(x) for x in fx["L"])
    rep = dict(L=L, n_fluid=0, n_mono=n, mol0_size=n, kT=float(fx["kT"]), shear=0.0, h=0.1,
               md_dt=float(fx["md_dt"]), seed=SEED, **{"lambda": float(fx["lam"])})
    nu = float(fx["andersen_nu"])
    o = orc.OracleSystem(L, float(fx["kT"]), 0.0, 1000, 0, n, mol_start=[0, n],
                         lambda_=float(fx["lam"]), md_dt=float(fx["md_dt"]))
    o.set_monomers(fx["mono_pos0"], fx["mono_vel0"], fx["mono_force0"], fx["mono_mass"],
                   fx["mono_amphi"], fx["mono_anchor"])
    o.set_bonds(fx["bond_src"], fx["bond_dst"])
    o.set_andersen(nu, SEED)
    o.init_md()
    with capi.Context([rep, rep], precision=capi.FP64, rng=capi.RNG_PHILOX, step_update=1000,
                      md_thermostat=capi.MDTHERMO_ANDERSEN, andersen_nu=nu) as ctx:
        for r in range(2):
            ctx.set_monomers(r, fx["mono_pos0"], fx["mono_vel0"], fx["mono_force0"],
                             fx["mono_mass"], fx["mono_amphi"], fx["mono_anchor"])
            ctx.set_bonds(r, fx["bond_src"], fx["bond_dst"])
        ctx.init_md()
        # a staged count that differs from the call's is refused, nothing runs
        ctx.stage_andersen(0, [0, 0, 0], [], np.zeros((0, 3)))
        with pytest.raises(capi.SmpcError):
            ctx.md_substeps(3)
        for t0 in range(0, 40, 4):
            starts, idx, vel = [0], [], []
            for t in range(t0, t0 + 4):
                i, v = gr.andersen_resets(fx, t)
                idx.append(i); vel.append(v)
                starts.append(starts[-1] + len(i))
                o.propagate(False)
            ctx.stage_andersen(0, starts, np.concatenate(idx), np.concatenate(vel))
            ctx.md_substeps(4)
        ctx.raise_on_device_error()
        p0, v0, _ = ctx.get_monomers(0)
        H.close64(p0, fx["mono_pos"][39])
        H.close64(v0, fx["mono_vel"][39])
        p1, v1, _ = ctx.get_monomers(1)
        op, ov, _ = o.get_monomers()
        H.close64(p1, op, rtol=1e-11)
        H.close64(v1, ov, rtol=1e-11)
        # out-of-range monomer, bad starts
        with pytest.raises(capi.SmpcError):
            ctx.stage_andersen(0, [0, 1], [n], np.zeros((1, 3)))
        with pytest.raises(capi.SmpcError):
            ctx.stage_andersen(0, [1, 1], [0], np.zeros((1, 3)))


def test_staging_needs_the_andersen_thermostat():
    L = 12
    star, _, _ = H.small_star_system(L=L, seed=6)
    n = star.n
    rep = dict(L=(L, L, L), n_fluid=0, n_mono=n, mol0_size=n, kT=1.0, shear=0.0, h=0.1,
               md_dt=0.01, **{"lambda": 1.0})
    with capi.Context([rep], precision=capi.FP64, rng=capi.RNG_PHILOX, step_update=1000) as ctx:
        with pytest.raises(capi.SmpcError):
            ctx.stage_andersen(0, [0, 0], [], np.zeros((0, 3)))


LOWE_NU, LOWE_R = 20.0, 1.5


def _lowe_pair(precision, seed=7, n_arm=8, arms=6, L=16):
    star, _, _ = H.small_star_system(L=L, n_c=1, arms=arms, n_arm=n_arm, seed=seed)
    n = star.n
    o = orc.OracleSystem((L, L, L), 1.0, 0.0, 1000, 0, n, mol_start=[0, n])
    o.set_monomers(star.pos, star.vel, np.zeros_like(star.pos), np.full(n, star.mass),
                   star.amphi, star.anchor)
    o.set_bonds(star.bond_src, star.bond_dst)
    o.set_lowe_andersen(LOWE_NU, LOWE_R, SEED)
    o.init_md()
    rep = dict(L=(L, L, L), n_fluid=0, n_mono=n, mol0_size=n, kT=1.0, shear=0.0, h=0.1,
               md_dt=0.01, seed=SEED, **{"lambda": 1.0})
    ctx = capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX, step_update=1000,
                       md_thermostat=capi.MDTHERMO_LOWE_ANDERSEN, andersen_nu=LOWE_NU,
                       lowe_radius=LOWE_R)
    ctx.set_monomers(0, star.pos, star.vel, np.zeros_like(star.pos), np.full(n, star.mass),
                     star.amphi, star.anchor)
    ctx.set_bonds(0, star.bond_src, star.bond_dst)
    ctx.init_md()
    return star, o, ctx


def test_fp64_lowe_andersen_matches_oracle():
    # the pair collisions in canonical order (beads ascending, partners
    # ascending) on the same Philox draws as the oracle's restatement of
    # Lowe_Andersen::propagate (Lowe_Andersen.cpp:46-88)
    star, o, ctx = _lowe_pair(capi.FP64)
    with ctx:
        before = ctx.get_monomers(0)[1].copy()
        for _ in range(40):
            o.propagate(False)
        ctx.md_substeps(25)
        ctx.md_substeps(15)
        ctx.raise_on_device_error()
        mp, mv, mf = ctx.get_monomers(0)
        op, ov, of = o.get_monomers()
        H.close64(mp, op, rtol=1e-11)
        H.close64(mv, ov, rtol=1e-11)
        H.close64(mf, of, rtol=1e-11)
        assert np.abs(mv - before).max() > 0.1  # the thermostat did act


@pytest.mark.parametrize("md_variant", [0, 2])
def test_fp32_lowe_andersen_conserves_momentum_and_holds_kT(md_variant):
    # md_variant 2 gives each bead several lanes (the candidates are still
    # taken by the bead's lead lane)
    star, o, ctx = _lowe_pair(capi.FP32, seed=9, n_arm=12, arms=8)
    with ctx:
        ctx.set_variants(0, 0, md_variant)
        m = star.mass
        p0 = m * ctx.get_monomers(0)[1].sum(axis=0)
        temps = []
        for _ in range(30):
            ctx.md_substeps(100)
            v = ctx.get_monomers(0)[1]
            u = v - v.mean(axis=0)
            temps.append(m * (u * u).sum() / (3 * (len(v) - 1)))
        ctx.raise_on_device_error()
        p1 = m * ctx.get_monomers(0)[1].sum(axis=0)
        scale = m * np.sqrt(len(v)) * 1.0 / np.sqrt(m)
        assert np.abs(p1 - p0).max() < 1e-3 * scale  # pairwise exchanges conserve momentum
        assert abs(np.mean(temps[5:]) - 1.0) < 0.12


def test_lowe_andersen_limits():
    # radius above r_cut, or a periodic box: refused at creation
    rep = dict(L=(12, 12, 12), n_fluid=0, n_mono=10, mol0_size=10, kT=1.0, md_dt=0.01,
               r_cut=1.5, r_verlet=2.0)
    with pytest.raises(capi.SmpcError):
        capi.Context([rep], precision=capi.FP64, rng=capi.RNG_PHILOX,
                     md_thermostat=capi.MDTHERMO_LOWE_ANDERSEN, andersen_nu=1.0, lowe_radius=1.8)
    per = dict(rep, flags=capi.REPLICA_PERIODIC_MD)
    with pytest.raises(capi.SmpcError):
        capi.Context([per], precision=capi.FP64, rng=capi.RNG_PHILOX,
                     mono_bin=capi.MONOBIN_WRAPPED,
                     md_thermostat=capi.MDTHERMO_LOWE_ANDERSEN, andersen_nu=1.0, lowe_radius=1.0)


LOWE_FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "lowe", "lowe_star.npz")


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32], ids=["fp64", "fp32"])
def test_lowe_andersen_statistics_match_reference(precision, record_property):
    # The reference's own Lowe_Andersen (Lowe_Andersen.cpp:46-88, nu = 20,
    # r = 1.5) in 8 independent runs of a 61-bead star with MPC off
    # (tests/golden/make_lowe.py) against 8 runs of the GPU's, as 8 replicas
    # in one context: bead temperature and the beads' normalised velocity
    # autocorrelation at 1..50 steps agree within 5 standard errors of the
    # difference (each from the spread of its runs); every run conserves the
    # total momentum (pairwise exchanges; round-off of the precision).
    if not os.path.exists(LOWE_FIXTURE):
        pytest.skip("Lowe-Andersen fixture not generated")
    fx = dict(np.load(LOWE_FIXTURE))
    ref = fx["runs"]
    n_runs, lags = len(ref), [int(x) for x in fx["lags"]]
    n = len(fx["star_pos"])
    L = int(fx["L"])
    reps = [dict(L=(L,) * 3, n_fluid=0, n_mono=n, mol0_size=n, kT=float(fx["kT"]), shear=0.0,
                 h=0.1, md_dt=float(fx["dt"]), seed=900 + 50 * precision + k,
                 **{"lambda": float(fx["lam"])}) for k in range(n_runs)]
    mass = fx["star_mass"]
    max_lag = max(lags)
    ring, sums, counts = [], np.zeros((n_runs, max_lag + 1)), np.zeros(max_lag + 1)
    t_sum = np.zeros(n_runs)
    pos = np.zeros((n_runs * n, 3))
    vel = np.zeros((n_runs * n, 3))
    with capi.Context(reps, precision=precision, rng=capi.RNG_PHILOX, step_update=1000,
                      md_thermostat=capi.MDTHERMO_LOWE_ANDERSEN, andersen_nu=float(fx["nu"]),
                      lowe_radius=float(fx["radius"])) as ctx:
        for k in range(n_runs):
            ctx.set_monomers(k, fx["star_pos"], fx["star_vel"], np.zeros_like(fx["star_pos"]),
                             mass, fx["star_amphi"], fx["star_anchor"])
            ctx.set_bonds(k, fx["bond_src"], fx["bond_dst"])
        ctx.init_md()
        ctx.md_substeps(int(fx["equil"]))
        p0 = None
        drift = np.zeros(n_runs)
        for _ in range(int(fx["steps"])):
            ctx.md_substeps(1)
            ctx.get_monomer_state_all(pos, vel)
            v = vel.reshape(n_runs, n, 3).copy()
            t_sum += (mass[None, :, None] * v * v).sum(axis=(1, 2)) / (3.0 * (n - 1))
            p = (mass[None, :, None] * v).sum(axis=1)
            if p0 is None:
                p0 = p
            drift = np.maximum(drift, np.abs(p - p0).max(axis=1))
            ring.append(v)
            if len(ring) > max_lag + 1:
                ring.pop(0)
            past = np.stack(ring[::-1])  # lag 0, 1, ...
            sums[:, : len(ring)] += np.einsum("lrnd,rnd->rl", past, v)
            counts[: len(ring)] += 1
        ctx.raise_on_device_error()
    c = sums / counts
    gpu = np.column_stack([t_sum / int(fx["steps"]), drift] +
                          [c[:, l] / c[:, 0] for l in lags])
    names = ["t_kin", "p_drift"] + [f"vacf_{l}" for l in lags]
    report = {}
    for j, name in enumerate(names):
        mg, sg = float(gpu[:, j].mean()), float(gpu[:, j].std(ddof=1) / np.sqrt(n_runs))
        mr, sr = float(ref[:, j].mean()), float(ref[:, j].std(ddof=1) / np.sqrt(n_runs))
        report[name] = (mg, mr, sg, sr)
    record_property("gpu_ref_mean_se", report)
    for name in names:
        if name == "p_drift":
            continue
        mg, mr, sg, sr = report[name]
        assert abs(mg - mr) < 5.0 * np.hypot(sg, sr), (name, report[name])
    p_scale = float(mass.sum()) * np.sqrt(float(fx["kT"]) / float(mass.mean()))
    assert drift.max() < (1e-11 if precision == capi.FP64 else 1e-4) * p_scale
