"""Parity of the CUDA path (through the C ABI) with the reference and the oracle.

FP64 path: bit-exact cell occupancies; positions, velocities, forces,
temperature and potential energy within 1e-12 of the reference (relative to
each array's scale), the Lees-Edwards offset bit-exact. FP32 path: stated
tolerances against the FP64 oracle on identical injected draws.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc
from starpolymersmd_gb300 import capi, system
from tests import golden_replay as gr
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

FIXTURES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_fp64_replays_reference_fixture(path):
    fx = gr.load(path)
    star = gr.has_star(fx)
    coll = gr.collision_index(fx)
    with H.fixture_context(fx) as ctx:
        if star:
            _, _, f0 = ctx.get_monomers(0)
            H.close64(f0, fx["mono_force0"])
        for t in range(int(fx["n_loop"])):
            if star and int(fx["with_md"]):
                if gr.is_andersen(fx):
                    idx, vel = gr.andersen_resets(fx, t)
                    ctx.stage_andersen(0, [0, len(idx)], idx, vel)
                ctx.md_substeps(1, calc_epot=True)
                H.close64(ctx.epot(0), fx["epot"][t])
            if not int(fx["md_only"]):
                k = coll.get(t)
                if k is not None:
                    ctx.mpc_step(t, float(fx["h"]), fx["shift"][k], np.nan_to_num(fx["gamma"][k]),
                                 fx["u_phi"][k], fx["u_theta"][k])
                    ctx.raise_on_device_error()
                    tot, fl = ctx.cell_counts(0)
                    np.testing.assert_array_equal(tot, fx["count_total"][k])
                    np.testing.assert_array_equal(fl, fx["count_fluid"][k])
                    fc, mc = ctx.cell_members(0)
                    np.testing.assert_array_equal(fc, fx["fluid_cell"][k])
                    np.testing.assert_array_equal(mc, fx["mono_cell"][k])
                    p, v = ctx.get_fluid(0)
                    H.close64(p, fx["fluid_pos"][k])
                    H.close64(v, fx["fluid_vel"][k])
                    H.close64(ctx.temperature(0), fx["temperature"][k])
                    if "observables" in fx:
                        # output-step observables and the VelocityX profile
                        H.close64(ctx.molecule_observables_all()[0], fx["observables"][k])
                        px, py = ctx.velocity_profile(0, float(fx["profile_width"]))
                        for got, want in ((px, fx["profile_x"][k]), (py, fx["profile_y"][k])):
                            np.testing.assert_array_equal(got[:, 2], want[:, 2])
                            H.close64(got[:, :2], want[:, :2])
                else:
                    ctx.mpc_step(t, float(fx["h"]))
            assert ctx.delrx(0) == fx["delrx"][t]
            if star:
                p, v, f = ctx.get_monomers(0)
                H.close64(p, fx["mono_pos"][t])
                H.close64(v, fx["mono_vel"][t])
                H.close64(f, fx["mono_force"][t], rtol=1e-11)
        ctx.raise_on_device_error()


@pytest.mark.parametrize("shear", [0.0, 0.05])
def test_fp64_philox_matches_oracle(shear):
    # production draws (Philox + Marsaglia-Tsang) on both sides, 3 cycles of
    # 10 MD substeps + 1 collision through the step-by-step API
    L, su, h = 10, 10, 0.1
    star, fpos, fvel = H.small_star_system(L=L, shear=shear)
    o = H.oracle_for(star, fpos, fvel, L, 1.0, shear, su)
    o.set_philox(seed=77, counter=5)
    with H.context_for(star, fpos, fvel, L, 1.0, shear, su, rng=capi.RNG_PHILOX, seed=77) as ctx:
        ctx.set_collision_counter(5)
        for t in range(0, 3 * su + 1):
            o.propagate(False)
            o.mpc_step(t, h)
            ctx.md_substeps(1)
            ctx.mpc_step(t, h)
        ctx.raise_on_device_error()
        assert o.error() == 0
        tot, fl = ctx.cell_counts(0)
        otot, ofl = o.cell_counts()
        np.testing.assert_array_equal(tot, otot)
        np.testing.assert_array_equal(fl, ofl)
        p, v = ctx.get_fluid(0)
        op, ov = o.get_fluid()
        H.close64(p, op)
        H.close64(v, ov)
        mp, mv, mf = ctx.get_monomers(0)
        omp, omv, omf = o.get_monomers()
        H.close64(mp, omp)
        H.close64(mv, omv)
        H.close64(ctx.temperature(0), o.temperature())
        assert ctx.delrx(0) == o.delrx


def test_fp64_graph_cycles_match_stepwise():
    # smpc_cycles (captured graph, device-side delrx and shift) against the
    # same cycles issued call by call
    L, su, h = 8, 10, 0.1
    star, fpos, fvel = H.small_star_system(L=L, shear=0.1, seed=5)
    kw = dict(rng=capi.RNG_PHILOX, seed=9)
    with H.context_for(star, fpos, fvel, L, 1.0, 0.1, su, **kw) as a, \
            H.context_for(star, fpos, fvel, L, 1.0, 0.1, su, **kw) as b:
        # call-by-call: cycles start right after a collision, so the first
        # cycle is t = 1..10 with the collision at t = 10
        for t in range(1, 3 * su + 1):
            a.md_substeps(1)
            a.mpc_step(t, h)
        b.cycles(3)
        b.synchronize()
        a.raise_on_device_error()
        b.raise_on_device_error()
        pa, va = a.get_fluid(0)
        pb, vb = b.get_fluid(0)
        H.close64(pb, pa)
        H.close64(vb, va)
        ma = a.get_monomers(0)
        mb = b.get_monomers(0)
        for x, y in zip(mb, ma):
            H.close64(x, y)
        assert a.delrx(0) == b.delrx(0)


@pytest.mark.parametrize("name", ["star_mpc_L12", "amc_star_L12"])
def test_fp32_matches_fp64_oracle_on_injected_draws(golden_dir, name):
    fx = gr.load(os.path.join(golden_dir, name + ".npz"))
    coll = gr.collision_index(fx)
    L = fx["L"]
    with H.fixture_context(fx, precision=capi.FP32) as ctx:
        for t in range(int(fx["n_loop"])):
            ctx.md_substeps(1)
            k = coll.get(t)
            if k is not None:
                ctx.mpc_step(t, float(fx["h"]), fx["shift"][k], np.nan_to_num(fx["gamma"][k]),
                             fx["u_phi"][k], fx["u_theta"][k])
                ctx.raise_on_device_error()
                p, v = ctx.get_fluid(0)
                dp = np.abs(H.wrapped_diff(p, fx["fluid_pos"][k], L)).max(axis=1)
                dv = np.abs(v - fx["fluid_vel"][k]).max(axis=1)
                vs = np.abs(fx["fluid_vel"][k]).max()
                # A particle within FP32 rounding of a cell face may land in the
                # neighbouring cell, which changes the collision of the two cells
                # involved; all other particles must agree to FP32 accuracy.
                bad = (dp > H.FP32_POS_ATOL * L.max()) | (dv > H.FP32_VEL_RTOL * vs)
                assert bad.mean() < 0.005, (bad.sum(), dp.max(), dv.max())
                tot, _ = ctx.cell_counts(0)
                assert np.count_nonzero(tot != fx["count_total"][k]) <= 4
                assert tot.sum() == fx["count_total"][k].sum()
            else:
                ctx.mpc_step(t, float(fx["h"]))
        mp, mv, _ = ctx.get_monomers(0)
        assert np.abs(mp - fx["mono_pos"][-1]).max() < 1e-3
        assert np.abs(mv - fx["mono_vel"][-1]).max() < 1e-2


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_collision_conserves_total_momentum(precision):
    # no shear, no recentring: streaming and shifting leave velocities alone
    # and every cell's collision conserves its momentum
    L = 12
    star, fpos, fvel = H.small_star_system(L=L, shear=0.0, seed=11, n_arm=4)
    with H.context_for(star, fpos, fvel, L, 1.0, 0.0, 1, rng=capi.RNG_PHILOX,
                       precision=precision) as ctx:
        m = star.mass

        def momentum():
            _, v = ctx.get_fluid(0)
            _, mv, _ = ctx.get_monomers(0)
            return v.sum(axis=0) + m * mv.sum(axis=0), np.abs(v).sum() + m * np.abs(mv).sum()

        p0, scale = momentum()
        for t in range(5):
            ctx.mpc_step(t, 0.1)
        ctx.raise_on_device_error()
        p1, _ = momentum()
        tol = 1e-12 if precision == capi.FP64 else 2e-6
        assert np.abs(p1 - p0).max() < tol * scale


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_thermostat_holds_temperature(precision):
    # MBS thermostat at kT = 1 from a cold start (uniform velocities, kT_init = 1/12)
    L = 10
    rng = np.random.default_rng(4)
    from starpolymersmd_gb300 import system
    fpos, fvel = system.uniform_fluid((L, L, L), 10, 1.0, rng, reference_velocities=True)
    rep = dict(L=(L, L, L), n_fluid=len(fpos), kT=1.0, shear=0.0, h=0.1, seed=21)
    with capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX, step_update=1) as ctx:
        ctx.set_fluid(0, fpos, fvel)
        temps = []
        for t in range(60):
            ctx.mpc_step(t, 0.1)
            if t >= 20:
                temps.append(ctx.temperature(0))
        ctx.raise_on_device_error()
        assert abs(np.mean(temps) - 1.0) < 0.01


def _batch_specs():
    from starpolymersmd_gb300 import system
    return [system.ReplicaSpec(L=9, arms=3, n_arm=5, solvophobic_fraction=0.4, shear=0.2, seed=31),
            system.ReplicaSpec(L=12, arms=4, n_arm=6, solvophobic_fraction=0.6, shear=0.01, seed=32),
            system.ReplicaSpec(L=7, arms=3, n_arm=3, solvophobic_fraction=0.5, shear=0.0, seed=33)]


def _batch_run(precision, cycles=2):
    """Uneven replicas in one context (production options) and one oracle per
    replica with the same options; returns both final states."""
    from starpolymersmd_gb300 import system, workloads as W
    specs = _batch_specs()
    stars, fluids, descs = [], [], []
    for s in specs:
        rng = np.random.default_rng(500 + s.seed)
        st = system.make_star(s.arms, s.n_arm, s.solvophobic_fraction, s.mono_mass, s.kT, rng,
                              bond=0.97)
        fp, fv = system.uniform_fluid((s.L,) * 3, s.n_c, s.kT, rng)
        stars.append(st)
        fluids.append((fp, fv))
        descs.append(W.replica_desc(s, st))
    ctx = capi.Context(descs, precision=precision, rng=capi.RNG_PHILOX,
                       mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL,
                       step_update=W.N_SUB, max_neighbors=W.MAX_NB, strict_cells=0)
    oracles = []
    for k, (s, st, (fp, fv)) in enumerate(zip(specs, stars, fluids)):
        ctx.set_fluid(k, fp, fv)
        ctx.set_monomers(k, st.pos, st.vel, np.zeros_like(st.pos), np.full(st.n, st.mass),
                         st.amphi, st.anchor)
        ctx.set_bonds(k, st.bond_src, st.bond_dst)
        o = orc.OracleSystem((s.L,) * 3, s.kT, s.shear, W.N_SUB, len(fp), st.n, mol_start=[0, st.n],
                             lambda_=1.0, md_dt=W.MD_DT, r_cut=W.R_CUT_LJ,
                             r_verlet=W.R_CUT_LJ + W.SKIN, potential=orc.POT_LJ126,
                             delrx_dt_scale=1.0 / W.N_SUB, mono_wrap=1)
        o.set_fluid(fp, fv)
        o.set_monomers(st.pos, st.vel, np.zeros_like(st.pos), np.full(st.n, st.mass), st.amphi,
                       st.anchor)
        o.set_bonds(st.bond_src, st.bond_dst)
        o.init_md()
        o.set_philox(s.seed, 0)
        oracles.append(o)
    ctx.init_md()
    ctx.cycles(cycles)
    ctx.synchronize()
    ctx.raise_on_device_error()
    for o in oracles:
        o.run(1, W.N_SUB * cycles, W.H, True)
        assert o.error() == 0
    return ctx, oracles, specs


def test_batched_fp64_matches_independent_oracles():
    ctx, oracles, specs = _batch_run(capi.FP64)
    with ctx:
        for k, (o, s) in enumerate(zip(oracles, specs)):
            tot, _ = ctx.cell_counts(k)
            otot, _ = o.cell_counts()
            np.testing.assert_array_equal(tot, otot)
            p, v = ctx.get_fluid(k)
            op, ov = o.get_fluid()
            H.close64(p, op)
            H.close64(v, ov)
            mp, mv, _ = ctx.get_monomers(k)
            omp, omv, _ = o.get_monomers()
            H.close64(mp, omp, rtol=1e-11)
            H.close64(mv, omv, rtol=1e-11)
            H.close64(ctx.temperature(k), o.temperature())
            assert ctx.delrx(k) == o.delrx


def test_batched_fp32_tracks_fp64_oracle():
    # FP32 state, fixed-point cell sums and FP32 Philox draws against the FP64
    # oracle consuming the same 23-bit uniforms, one cycle at a time from the
    # FP32 state: every particle outside the cells where a particle within
    # FP32 rounding of a face was binned differently agrees to FP32 accuracy
    # (tests/gpu_helpers.fp32_cycle_check).
    ctx, oracles, specs = _batch_run(capi.FP32, cycles=0)
    for o in oracles:
        o.set_f32_uniforms(True)
    with ctx:
        from starpolymersmd_gb300 import workloads as W
        for c in range(3):
            for k, o in enumerate(oracles):
                H.resync_oracle(ctx, o, k)
            ctx.cycles(1)
            ctx.synchronize()
            ctx.raise_on_device_error()
            for k, (o, s) in enumerate(zip(oracles, specs)):
                o.run(1 + W.N_SUB * c, W.N_SUB, W.H, True)
                assert o.error() == 0
                H.fp32_cycle_check(ctx, o, k, s.L)
                # the fast path's cell-ordered records give the same membership as its counts
                tot, fl = ctx.cell_counts(k)
                fc, mc = ctx.cell_members(k)
                n = len(tot)
                np.testing.assert_array_equal(np.bincount(fc, minlength=n), fl)
                np.testing.assert_array_equal(np.bincount(fc, minlength=n) +
                                              np.bincount(mc[mc >= 0], minlength=n), tot)


def test_fp32_launch_variants_agree_bitwise():
    # Every launch shape of the fast-path solvent kernels gives the same
    # solvent state to the last bit: cell sums are int64 fixed point
    # (independent of particle order) and each particle's update is a pure
    # function of its cell's sums and draws.
    from starpolymersmd_gb300 import system
    rng = np.random.default_rng(8)
    reps, states = [], []
    for k, L in enumerate((11, 14)):
        fp, fv = system.uniform_fluid((L, L, L), 10, 1.0, rng)
        reps.append(dict(L=(L, L, L), n_fluid=len(fp), kT=1.0, shear=0.02 * (k + 1), h=0.1,
                         seed=40 + k))
        states.append((fp, fv))
    finals = []
    lib = capi.load()
    n_bin, n_col = 4, 12
    for vb, vc in [(0, 0)] + [(b, 0) for b in range(1, n_bin)] + [(0, c) for c in range(1, n_col)]:
        with capi.Context(reps, precision=capi.FP32, rng=capi.RNG_PHILOX, step_update=1,
                          strict_cells=0) as ctx:
            for k, (fp, fv) in enumerate(states):
                ctx.set_fluid(k, fp, fv)
            ctx.set_variants(vb, vc, 0)
            ctx.cycles(3)
            ctx.synchronize()
            ctx.raise_on_device_error()
            finals.append([ctx.get_fluid(k) for k in range(len(reps))])
    for other in finals[1:]:
        for (p0, v0), (p1, v1) in zip(finals[0], other):
            np.testing.assert_array_equal(p0, p1)
            np.testing.assert_array_equal(v0, v1)


def test_fp32_packed_and_wide_sort_keys_agree_bitwise():
    # Contexts whose boxes all have at most 65,536 cells sort with 32-bit keys
    # (local cell << 16 | rank); a box of 41^3 cells sends its context to the
    # (global cell, rank) pairs. The 12^3 box evolves to the same bits either way.
    from starpolymersmd_gb300 import system
    rng = np.random.default_rng(21)
    small = system.uniform_fluid((12, 12, 12), 10, 1.0, rng)
    big = system.uniform_fluid((41, 41, 41), 10, 1.0, rng)
    reps = [dict(L=(12, 12, 12), n_fluid=len(small[0]), kT=1.0, shear=0.05, h=0.1, seed=7),
            dict(L=(41, 41, 41), n_fluid=len(big[0]), kT=1.0, shear=0.02, h=0.1, seed=8)]
    kw = dict(precision=capi.FP32, rng=capi.RNG_PHILOX, step_update=1, strict_cells=0)
    out = []
    for rs, states in ((reps[:1], [small]), (reps, [small, big])):
        with capi.Context(rs, **kw) as ctx:
            for k, (fp, fv) in enumerate(states):
                ctx.set_fluid(k, fp, fv)
            ctx.cycles(3)
            ctx.raise_on_device_error()
            out.append(ctx.get_fluid(0))
            tot, fl = ctx.cell_counts(0)
            fc, _ = ctx.cell_members(0)
            np.testing.assert_array_equal(np.bincount(fc, minlength=len(tot)), fl)
    for x, y in zip(*out):
        np.testing.assert_array_equal(x, y)


def test_fp32_collide_variants_agree_bitwise_with_stars():
    # the same with monomers in the cells (staged from the monomer arrays,
    # written back to them), MD substeps in between
    finals = []
    for vc in range(12):
        ctx, _, specs = _batch_run(capi.FP32, cycles=0)
        with ctx:
            ctx.set_variants(0, vc, 0)
            ctx.cycles(3)
            ctx.synchronize()
            ctx.raise_on_device_error()
            finals.append([ctx.get_fluid(k) + ctx.get_monomers(k)[:2] for k in range(len(specs))])
    for other in finals[1:]:
        for a, b in zip(finals[0], other):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y)


def test_autotune_reports_and_keeps_a_variant():
    from starpolymersmd_gb300 import system
    rng = np.random.default_rng(9)
    fp, fv = system.uniform_fluid((12, 12, 12), 10, 1.0, rng)
    rep = dict(L=(12, 12, 12), n_fluid=len(fp), kT=1.0, shear=0.05, h=0.1, seed=5)
    with capi.Context([rep], precision=capi.FP32, rng=capi.RNG_PHILOX, step_update=1,
                      strict_cells=0) as ctx:
        ctx.set_fluid(0, fp, fv)
        report = ctx.autotune(2)
        assert set(report) == {"fluid_bin", "collide", "md_substeps"}
        chosen = ctx.get_variants()
        assert chosen[0] == report["fluid_bin"]["index"]
        assert chosen[1] == report["collide"]["index"]
        ctx.cycles(2)
        ctx.raise_on_device_error()
        assert abs(ctx.temperature(0) - 1.0) < 0.2


@pytest.mark.parametrize("md_variant", [0, 1, 2, 3, 4])
def test_fp32_md_variants_are_reproducible(md_variant):
    # two runs of the same replicas give the same bits: the Verlet lists come
    # out in the same order whatever order the hash-grid insertions ran in
    # (stars of 16 to 121 beads, so a replica spans several warps)
    from starpolymersmd_gb300 import system, workloads as W
    specs = _batch_specs() + [system.ReplicaSpec(L=14, arms=6, n_arm=20, solvophobic_fraction=0.5,
                                                 shear=0.05, seed=34)]
    descs, states = [], []
    for s in specs:
        rng = np.random.default_rng(900 + s.seed)
        st = system.make_star(s.arms, s.n_arm, s.solvophobic_fraction, s.mono_mass, s.kT, rng,
                              bond=0.97)
        descs.append(W.replica_desc(s, st))
        states.append((st, system.uniform_fluid((s.L,) * 3, s.n_c, s.kT, rng)))
    kw = dict(precision=capi.FP32, rng=capi.RNG_PHILOX, mono_bin=capi.MONOBIN_WRAPPED,
              delrx_mode=capi.DELRX_PHYSICAL, step_update=W.N_SUB, max_neighbors=W.MAX_NB,
              strict_cells=0)
    runs = []
    for _ in range(2):
        with capi.Context(descs, **kw) as ctx:
            ctx.set_variants(0, 0, md_variant)
            for k, (st, (fp, fv)) in enumerate(states):
                ctx.set_fluid(k, fp, fv)
                ctx.set_monomers(k, st.pos, st.vel, np.zeros_like(st.pos),
                                 np.full(st.n, st.mass), st.amphi, st.anchor)
                ctx.set_bonds(k, st.bond_src, st.bond_dst)
            ctx.init_md()
            ctx.cycles(4)
            ctx.raise_on_device_error()
            runs.append([ctx.get_fluid(k) + ctx.get_monomers(k) for k in range(len(specs))])
    for a, b in zip(*runs):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


def test_autotune_leaves_the_trajectory_where_it_was():
    # the autotuner's trial cycles run on a saved copy of the state: a context
    # that tunes between two stretches of cycles ends with the same bits as
    # one that only switches to the chosen variants at the same point
    from starpolymersmd_gb300 import system, workloads as W
    specs = _batch_specs()
    descs, states = [], []
    for s in specs:
        rng = np.random.default_rng(700 + s.seed)
        st = system.make_star(s.arms, s.n_arm, s.solvophobic_fraction, s.mono_mass, s.kT, rng,
                              bond=0.97)
        descs.append(W.replica_desc(s, st))
        states.append((st, system.uniform_fluid((s.L,) * 3, s.n_c, s.kT, rng)))
    kw = dict(precision=capi.FP32, rng=capi.RNG_PHILOX, mono_bin=capi.MONOBIN_WRAPPED,
              delrx_mode=capi.DELRX_PHYSICAL, step_update=W.N_SUB, max_neighbors=W.MAX_NB,
              strict_cells=0)
    with capi.Context(descs, **kw) as a, capi.Context(descs, **kw) as b:
        for ctx in (a, b):
            for k, (st, (fp, fv)) in enumerate(states):
                ctx.set_fluid(k, fp, fv)
                ctx.set_monomers(k, st.pos, st.vel, np.zeros_like(st.pos),
                                 np.full(st.n, st.mass), st.amphi, st.anchor)
                ctx.set_bonds(k, st.bond_src, st.bond_dst)
            ctx.init_md()
            ctx.cycles(3)
        a.autotune(2)
        b.set_variants(*a.get_variants())
        a.cycles(3)
        b.cycles(3)
        a.raise_on_device_error()
        b.raise_on_device_error()
        for k in range(len(specs)):
            for x, y in zip(a.get_fluid(k), b.get_fluid(k)):
                np.testing.assert_array_equal(x, y)
            for x, y in zip(a.get_monomers(k), b.get_monomers(k)):
                np.testing.assert_array_equal(x, y)
            assert a.delrx(k) == b.delrx(k)


@pytest.mark.parametrize("name", ["star_mpc_L12", "mpc_shear_L6"])
def test_two_phase_step_replays_reference(golden_dir, name):
    # smpc_mpc_bin with the reference's grid shift, occupancies read back
    # between the phases (what decides which cells draw a gamma variate), then
    # smpc_mpc_collide with the reference's per-cell draws.
    fx = gr.load(os.path.join(golden_dir, name + ".npz"))
    coll = gr.collision_index(fx)
    star = gr.has_star(fx)
    with H.fixture_context(fx) as ctx:
        for t in range(int(fx["n_loop"])):
            if star and int(fx["with_md"]):
                ctx.md_substeps(1)
            k = coll.get(t)
            binned = ctx.mpc_bin(t, float(fx["h"]), None if k is None else fx["shift"][k])
            assert binned == (k is not None)
            if binned:
                tot, fl = ctx.cell_counts(0)
                np.testing.assert_array_equal(tot, fx["count_total"][k])
                np.testing.assert_array_equal(fl, fx["count_fluid"][k])
                with pytest.raises(capi.SmpcError):
                    ctx.cell_members(0)  # records are reordered only by the collision
                ctx.mpc_collide(np.nan_to_num(fx["gamma"][k]), fx["u_phi"][k], fx["u_theta"][k])
                ctx.raise_on_device_error()
                fc, mc = ctx.cell_members(0)
                np.testing.assert_array_equal(fc, fx["fluid_cell"][k])
                np.testing.assert_array_equal(mc, fx["mono_cell"][k])
                p, v = ctx.get_fluid(0)
                H.close64(p, fx["fluid_pos"][k])
                H.close64(v, fx["fluid_vel"][k])
            assert ctx.delrx(0) == fx["delrx"][t]


@pytest.mark.parametrize("md_variant", [0, 1, 2, 3, 4])
def test_fp32_md_variants_track_fp64_oracle(md_variant):
    # MD only (no collisions): every FP32 launch shape of the substep kernel,
    # including the one that splits a bead's Verlet list over several lanes,
    # the one that runs stars above 512 beads in a second kernel beside the
    # rest and the one that spreads each replica over a cluster of SMs,
    # follows the FP64 oracle to FP32 round-off over 20 substeps.
    from starpolymersmd_gb300 import system, workloads as W
    specs = _batch_specs() + [system.ReplicaSpec(L=16, arms=6, n_arm=20, solvophobic_fraction=0.3,
                                                 shear=0.05, seed=34),
                              system.ReplicaSpec(L=28, arms=12, n_arm=45,
                                                 solvophobic_fraction=0.5, shear=0.02, seed=35)]
    assert max(s.arms * s.n_arm + 1 for s in specs) > 512
    stars, descs = [], []
    for s in specs:
        st = system.make_star(s.arms, s.n_arm, s.solvophobic_fraction, s.mono_mass, s.kT,
                              np.random.default_rng(600 + s.seed), bond=0.97)
        stars.append(st)
        descs.append(W.replica_desc(s, st))
    n_sub = 20
    with capi.Context(descs, precision=capi.FP32, rng=capi.RNG_PHILOX,
                      mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL,
                      step_update=W.N_SUB, max_neighbors=W.MAX_NB, strict_cells=0) as ctx:
        ctx.set_variants(0, 0, md_variant)
        for k, st in enumerate(stars):
            ctx.set_monomers(k, st.pos, st.vel, np.zeros_like(st.pos), np.full(st.n, st.mass),
                             st.amphi, st.anchor)
            ctx.set_bonds(k, st.bond_src, st.bond_dst)
        ctx.init_md()
        ctx.md_substeps(n_sub)
        ctx.raise_on_device_error()
        for k, (s, st) in enumerate(zip(specs, stars)):
            o = orc.OracleSystem((s.L,) * 3, s.kT, s.shear, W.N_SUB, 0, st.n, mol_start=[0, st.n],
                                 lambda_=1.0, md_dt=W.MD_DT, r_cut=W.R_CUT_LJ,
                                 r_verlet=W.R_CUT_LJ + W.SKIN, potential=orc.POT_LJ126,
                                 delrx_dt_scale=1.0 / W.N_SUB, mono_wrap=1)
            o.set_monomers(st.pos, st.vel, np.zeros_like(st.pos), np.full(st.n, st.mass),
                           st.amphi, st.anchor)
            o.set_bonds(st.bond_src, st.bond_dst)
            o.init_md()
            for _ in range(n_sub):
                o.propagate(False)
            assert o.error() == 0
            mp, mv, mf = ctx.get_monomers(k)
            op, ov, of = o.get_monomers()
            np.testing.assert_allclose(mp, op, atol=1e-4)
            np.testing.assert_allclose(mv, ov, atol=2e-3 * np.abs(ov).max())
            np.testing.assert_allclose(mf, of, atol=2e-3 * np.abs(of).max())


def _numpy_observables(pos, vel, mass, mol_start):
    """The reference's output-step observables (Box.cpp:81-102, 288-294,
    330-379, 635-646) restated in numpy for one replica."""
    rg, G, w, ekin = 0.0, np.zeros((3, 3)), np.zeros(3), 0.0
    for a, b in zip(mol_start[:-1], mol_start[1:]):
        r = pos[a:b] - pos[a:b].mean(axis=0)
        u = vel[a:b] - vel[a:b].mean(axis=0)
        g = r.T @ r / (b - a)
        G += g
        rg += np.sqrt(np.trace(g))
        S = r.T @ r
        w += np.linalg.solve(np.trace(S) * np.eye(3) - S, np.cross(r, u).sum(axis=0))
        ekin += 0.5 * (mass[a:b] * (u * u).sum(axis=1)).sum()
    nm = len(mol_start) - 1
    n = mol_start[-1]
    return np.concatenate([[rg / nm], (G / nm).ravel(), w / nm, [ekin, ekin * 2 / (3 * (n - 1)), nm]])


def _numpy_profile(fpos, fvel, c_pos, c_vel, L, shear, delrx, width):
    p = fpos - c_pos
    v = fvel - c_vel
    cy = np.round(p[:, 1] / L[1]) if shear != 0 else np.zeros(len(p))
    if shear != 0:
        p[:, 0] -= L[0] * np.round(p[:, 0] / L[0])
        p[:, 0] -= cy * delrx
        p[:, 0] -= L[0] * np.round(p[:, 0] / L[0])
        p[:, 1] -= L[1] * cy
        v[:, 0] -= cy * shear * L[1]
    else:
        p[:, 0] -= np.round(p[:, 0] / L[0]) * L[0]
        p[:, 1] -= np.round(p[:, 1] / L[1]) * L[1]
    out = []
    for ax in (0, 1):
        k0 = np.floor(-L[ax] / (2 * width))
        k = (np.floor(p[:, ax] / width) - k0).astype(int)
        n = capi.profile_bins(L[ax], width)
        prof = np.zeros((n, 3))
        np.add.at(prof[:, 0], k, v[:, 0])
        np.add.at(prof[:, 1], k, v[:, 1])
        np.add.at(prof[:, 2], k, 1.0)
        out.append(prof)
    return out


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_observables_of_every_replica_match_numpy(precision):
    # batched layout (monomer offsets per replica), molecules set by the
    # caller, both precisions: the device observables against a numpy
    # restatement of the reference's definitions on the same state
    ctx, _, specs = _batch_run(precision, cycles=1)
    with ctx:
        n1 = None
        for k, s in enumerate(specs):
            if k == 1:  # split replica 1's star into two molecules
                n = ctx.replicas[k]["n_mono"]
                n1 = n // 3
                ctx.set_molecules(k, [0, n1, n])
        obs = ctx.molecule_observables_all()
        width = 0.2
        for k, s in enumerate(specs):
            pos, vel, _ = ctx.get_monomers(k)
            mass = np.full(len(pos), s.mono_mass)
            n = len(pos)
            ms = [0, n1, n] if k == 1 else [0, n]
            want = _numpy_observables(pos, vel, mass, ms)
            tol = 1e-9 if precision == capi.FP64 else 1e-5
            np.testing.assert_allclose(obs[k], want, rtol=tol, atol=tol * np.abs(want).max())
            fp, fv = ctx.get_fluid(k)
            L = (s.L,) * 3
            px, py = ctx.velocity_profile(k, width)
            c_pos, c_vel = pos[:ms[1]].mean(axis=0), vel[:ms[1]].mean(axis=0)
            wx, wy = _numpy_profile(fp, fv, c_pos, c_vel, L, s.shear, ctx.delrx(k), width)
            for got, want_p in ((px, wx), (py, wy)):
                # a particle within rounding of a bin face may fall on either side
                assert np.abs(got[:, 2] - want_p[:, 2]).sum() <= 4
                assert abs(got[:, 2].sum() - len(fp)) == 0
                np.testing.assert_allclose(got[:, :2].sum(axis=0), want_p[:, :2].sum(axis=0),
                                           rtol=1e-6, atol=1e-6 * len(fp))


@pytest.mark.parametrize("offset", [0.0, 2.6])
def test_fp32_graph_cycles_match_stepwise(offset):
    # FP32 fast path: graph cycles (delrx and grid shift advanced on the
    # device) against the same cycles issued call by call (host delrx): the
    # same state to the last bit. With the star moved next to the box face,
    # check_bounds recentres it inside the cycles.
    L, su, h = 10, 10, 0.1
    star, fpos, fvel = H.small_star_system(L=L, shear=0.1, seed=5)
    star.pos[:] += offset
    kw = dict(rng=capi.RNG_PHILOX, seed=9, precision=capi.FP32, strict=0,
              mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL)
    with H.context_for(star, fpos, fvel, L, 1.0, 0.1, su, **kw) as a, \
            H.context_for(star, fpos, fvel, L, 1.0, 0.1, su, **kw) as b:
        for t in range(1, 4 * su + 1):
            a.md_substeps(1)
            a.mpc_step(t, h)
        b.cycles(4)
        b.synchronize()
        a.raise_on_device_error()
        b.raise_on_device_error()
        pa, va = a.get_fluid(0)
        pb, vb = b.get_fluid(0)
        np.testing.assert_array_equal(pb, pa)
        np.testing.assert_array_equal(vb, va)
        for x, y in zip(b.get_monomers(0), a.get_monomers(0)):
            np.testing.assert_array_equal(x, y)
        # call-by-call cycles between graph cycles: the host's delrx mirror
        # and the device state stay in step
        for t in range(4 * su + 1, 6 * su + 1):
            a.md_substeps(1)
            a.mpc_step(t, h)
        for t in range(4 * su + 1, 5 * su + 1):
            b.md_substeps(1)
            b.mpc_step(t, h)
        b.cycles(1)
        b.synchronize()
        for x, y in zip(b.get_fluid(0), a.get_fluid(0)):
            np.testing.assert_array_equal(x, y)


def test_fp32_side_by_side_md_in_graph_cycles():
    # The side-by-side MD shape (stars above 512 beads on a forked stream,
    # joined before the collision) inside captured cycles, against the
    # single-kernel lanes-per-bead shape. The FP32 MD sums forces in the order
    # its shared-memory cell lists come out, so runs agree to FP32 round-off,
    # not bit for bit: every box, big, mid-sized and small, must follow.
    from starpolymersmd_gb300 import system, workloads as W
    specs = [system.ReplicaSpec(L=28, arms=12, n_arm=45, solvophobic_fraction=0.5, shear=0.02,
                                seed=41),
             system.ReplicaSpec(L=16, arms=8, n_arm=20, solvophobic_fraction=0.4, shear=0.05,
                                seed=42),
             system.ReplicaSpec(L=10, arms=4, n_arm=10, solvophobic_fraction=0.5, shear=0.1,
                                seed=43)]
    sizes = [s.arms * s.n_arm + 1 for s in specs]
    assert sizes[0] > 512 and 64 < sizes[1] <= 512 and sizes[2] <= 64
    a, b = W.build(specs), W.build(specs)
    try:
        a.ctx.set_variants(0, 5, 2)
        b.ctx.set_variants(0, 5, 3)
        for x in (a, b):
            x.ctx.cycles(3)
            x.ctx.synchronize()
            x.ctx.raise_on_device_error()
        for k, s in enumerate(specs):
            L = (s.L,) * 3
            (pa, va, _), (pb, vb, _) = a.ctx.get_monomers(k), b.ctx.get_monomers(k)
            assert np.abs(H.wrapped_diff(pa, pb, L)).max() < 1e-3
            assert np.abs(va - vb).max() < 1e-2 * np.abs(va).max()
            (fpa, fva), (fpb, fvb) = a.ctx.get_fluid(k), b.ctx.get_fluid(k)
            assert np.abs(H.wrapped_diff(fpa, fpb, L)).max() < 1e-3
            assert np.abs(fva - fvb).max() < 1e-2 * np.abs(fva).max()
    finally:
        a.close()
        b.close()


def test_cycles_io_is_the_separate_calls():
    # smpc_cycles_io = set state, cycles, get state, observables with one
    # synchronisation: two contexts from the same inputs, one through the
    # separate calls and one through the fused call (FP64: the MD sums are
    # in a fixed order, so the runs agree bit for bit up to the atomics of
    # the cell sort, which only permute particles inside a cell)
    from starpolymersmd_gb300 import workloads as W
    specs = _batch_specs()
    a, b = W.build(specs, precision=capi.FP64), W.build(specs, precision=capi.FP64)
    try:
        n = int(sum(a.n_mono))
        pa, va = np.zeros((n, 3)), np.zeros((n, 3))
        a.ctx.get_monomer_state_all(pa, va)
        va *= 0.9  # a state change the upload must carry
        pb, vb = pa.copy(), va.copy()
        a.ctx.set_monomer_state_all(pa, va)
        a.ctx.cycles(2)
        a.ctx.get_monomer_state_all(pa, va)
        obs_a = a.ctx.molecule_observables_all()
        obs_b = np.zeros_like(obs_a)
        b.ctx.cycles_io(2, pb, vb, pb, vb, obs_b)
        for x in (a, b):
            x.ctx.raise_on_device_error()
        H.close64(pb, pa)
        H.close64(vb, va)
        H.close64(obs_b, obs_a)
        # outputs only, and inputs only
        p2, v2 = np.zeros((n, 3)), np.zeros((n, 3))
        b.ctx.cycles_io(0, None, None, p2, v2, None)
        np.testing.assert_array_equal(p2, pb)
        with pytest.raises(capi.SmpcError):
            b.ctx.cycles_io(1, pb, None, None, None, None)
    finally:
        a.close()
        b.close()


def test_cycles_io_pinned_input_is_read_in_place():
    # pinned host arrays are read by the unpack kernel over the C2C link; the
    # result must equal the staged upload of the same (pageable) arrays
    torch = pytest.importorskip("torch")
    from starpolymersmd_gb300 import workloads as W
    specs = _batch_specs()
    a, b = W.build(specs, precision=capi.FP64), W.build(specs, precision=capi.FP64)
    try:
        n = int(sum(a.n_mono))
        p, v = np.zeros((n, 3)), np.zeros((n, 3))
        a.ctx.get_monomer_state_all(p, v)
        v *= 1.1
        pp = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        vp = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        pp[:], vp[:] = p, v
        a.ctx.cycles_io(0, p, v, None, None, None)       # pageable: staged copy
        b.ctx.cycles_io(0, pp, vp, None, None, None)     # pinned: read in place
        for x in (a, b):
            x.ctx.raise_on_device_error()
        qa, wa = np.zeros((n, 3)), np.zeros((n, 3))
        qb, wb = np.zeros((n, 3)), np.zeros((n, 3))
        a.ctx.get_monomer_state_all(qa, wa)
        b.ctx.get_monomer_state_all(qb, wb)
        np.testing.assert_array_equal(qa, qb)
        np.testing.assert_array_equal(wa, wb)
        np.testing.assert_array_equal(wa, v)  # FP64 state: the upload is exact
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("md_variant", [0, 1], ids=["cluster", "one_cta"])
def test_fp64_md_shapes_match_oracle(md_variant):
    # FP64 contexts of few replicas run each replica's MD on a cluster of SMs
    # (variant 0); variant 1 keeps one CTA per replica. Both follow the
    # oracle at 1e-12 over 3 cycles of the config-1 star with Andersen-free
    # velocity Verlet, with and without an energy read-out.
    L, su, h = 20, 10, 0.1
    star, fpos, fvel = H.small_star_system(L=L, arms=6, n_arm=20, shear=0.05, seed=1)
    o = H.oracle_for(star, fpos, fvel, L, 1.0, 0.05, su)
    o.set_philox(seed=5, counter=0)
    with H.context_for(star, fpos, fvel, L, 1.0, 0.05, su, rng=capi.RNG_PHILOX, seed=5) as ctx:
        ctx.set_variants(0, 0, md_variant)
        for t in range(0, 3 * su + 1):
            o.propagate(t == 3 * su)
            o.mpc_step(t, h)
            ctx.md_substeps(1, calc_epot=(t == 3 * su))
            ctx.mpc_step(t, h)
        ctx.raise_on_device_error()
        assert o.error() == 0
        mp, mv, mf = ctx.get_monomers(0)
        omp, omv, omf = o.get_monomers()
        H.close64(mp, omp)
        H.close64(mv, omv)
        H.close64(mf, omf, rtol=1e-11)
        H.close64(ctx.epot(0), o.epot())
        p, v = ctx.get_fluid(0)
        op, ov = o.get_fluid()
        H.close64(p, op)
        H.close64(v, ov)
        assert ctx.verlet_rebuilds(0) >= 1


@pytest.mark.parametrize("L,shear", [(7, 0.0), (20, 0.3), (29, 0.05)])
def test_fp64_wraps_bitwise_at_the_faces(L, shear):
    # The FP64 kernels decide each wrap's image from the magnitude bits of
    # the coordinate instead of round(x / L); solvent particles at rest
    # exactly on, and a few ulps either side of, +-L/2 and +-1.5 L (and 2.5 L)
    # on every axis must come out of a collision (stream, shift, sort,
    # unshift, with the reference's LEBC at every step) bit for bit as the
    # oracle's, which evaluates the reference's formula.
    rng = np.random.default_rng(L)
    base = []
    for edge in (0.5, 1.5):
        for k in range(-4, 5):
            e = edge * L * (1.0 + k * 2.0 ** -52)
            base += [e, -e, np.nextafter(e, 0.0), np.nextafter(-e, 0.0)]
    base += [2.5 * L, -2.5 * L, 0.0]
    vals = np.array(base)
    pts = []
    for ax in range(3):
        for v in vals:
            p = (rng.random(3) - 0.5) * 0.5 * L
            p[ax] = v
            pts.append(p)
    edge_pos = np.array(pts)
    fpos, fvel = system.uniform_fluid((L, L, L), 10, 1.0, rng)
    fpos = np.concatenate([fpos, edge_pos])
    fvel = np.concatenate([fvel, np.zeros_like(edge_pos)])
    n_cell = L ** 3
    # nonzero shifts: binning happens away from the faces (points a few ulps
    # inside +L/2 would otherwise hit the reference's own cell aliasing), while
    # the streaming and the unshift wrap at the edges themselves
    for shift in (np.array([0.25, -0.125, 0.375]), np.array([-0.3, 0.45, -0.05])):
        inj = (shift, rng.gamma(13.5, 1.0, n_cell), rng.random(n_cell), rng.random(n_cell))
        o = orc.OracleSystem((L,) * 3, 1.0, shear, 1, len(fpos))
        o.delrx = 0.3 * L
        o.set_fluid(fpos, fvel)
        o.set_inject(*inj)
        o.mpc_step(0, 0.1)
        assert o.error() == 0
        rep = dict(L=(L,) * 3, n_fluid=len(fpos), kT=1.0, shear=shear, h=0.1)
        with capi.Context([rep], precision=capi.FP64, rng=capi.RNG_INJECT, step_update=1) as ctx:
            ctx.set_delrx(0, 0.3 * L)
            ctx.set_fluid(0, fpos, fvel)
            ctx.mpc_step(0, 0.1, *inj)
            ctx.raise_on_device_error()
            p, v = ctx.get_fluid(0)
            op, ov = o.get_fluid()
            np.testing.assert_array_equal(p, op)
            fc, _ = ctx.cell_members(0)
            ofc, _ = o.cell_members()
            np.testing.assert_array_equal(fc, ofc)
            H.close64(v, ov)
            assert ctx.delrx(0) == o.delrx


def test_fp32_graph_cycles_after_host_solvent_change():
    # FP32 graph cycles must see a host change of the solvent between calls
    # (the captured graph reads the device buffers the upload wrote). Context
    # b runs 3 cycles, gets a new solvent state for replica 0, runs 3 more;
    # context c starts from exactly that state (same counters, delrx, other
    # replica) and runs 3: the same bits.
    rng = np.random.default_rng(17)
    reps, states = [], []
    for k, L in enumerate((9, 12)):
        fp, fv = system.uniform_fluid((L, L, L), 10, 1.0, rng)
        reps.append(dict(L=(L, L, L), n_fluid=len(fp), kT=1.0, shear=0.05 * (k + 1), h=0.1,
                         seed=70 + k))
        states.append((fp, fv))
    new0 = system.uniform_fluid((9, 9, 9), 10, 1.0, rng)
    kw = dict(precision=capi.FP32, rng=capi.RNG_PHILOX, step_update=1, strict_cells=0)
    with capi.Context(reps, **kw) as b, capi.Context(reps, **kw) as c:
        for k, (fp, fv) in enumerate(states):
            b.set_fluid(k, fp, fv)
        b.cycles(3)
        b.set_fluid(0, *new0)
        mid1 = b.get_fluid(1)
        c.set_fluid(0, *new0)
        c.set_fluid(1, *mid1)
        for k in range(2):
            c.set_delrx(k, b.delrx(k))
        c.set_collision_counter(3)
        b.cycles(3)
        c.cycles(3)
        b.raise_on_device_error()
        c.raise_on_device_error()
        for k in range(2):
            for x, y in zip(b.get_fluid(k), c.get_fluid(k)):
                np.testing.assert_array_equal(x, y)


def test_fp32_graph_cycles_with_recentring_in_one_replica():
    # two boxes in one context, graph cycles against call-by-call cycles:
    # replica 0's star sits at the box face so MPC::check_bounds recentres it,
    # replica 1's does not -- the same bits for both
    L, su, h = 10, 10, 0.1
    systems = [H.small_star_system(L=L, shear=0.1, seed=5), H.small_star_system(L=L, shear=0.05, seed=6)]
    systems[0][0].pos[:] += 2.6
    reps = [dict(L=(L,) * 3, n_fluid=len(fp), n_mono=st.n, mol0_size=st.n, kT=1.0, shear=sh,
                 h=h, md_dt=0.01, seed=9 + k)
            for k, ((st, fp, fv), sh) in enumerate(zip(systems, (0.1, 0.05)))]
    kw = dict(precision=capi.FP32, rng=capi.RNG_PHILOX, step_update=su, strict_cells=0,
              mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL)
    with capi.Context(reps, **kw) as a, capi.Context(reps, **kw) as b:
        for ctx in (a, b):
            for k, (st, fp, fv) in enumerate(systems):
                ctx.set_fluid(k, fp, fv)
                ctx.set_monomers(k, st.pos, st.vel, np.zeros_like(st.pos), np.full(st.n, st.mass),
                                 st.amphi, st.anchor)
                ctx.set_bonds(k, st.bond_src, st.bond_dst)
            ctx.init_md()
        for t in range(1, 4 * su + 1):
            a.md_substeps(1)
            a.mpc_step(t, h)
        b.cycles(4)
        b.synchronize()
        a.raise_on_device_error()
        b.raise_on_device_error()
        for k in range(2):
            for x, y in zip(b.get_fluid(k), a.get_fluid(k)):
                np.testing.assert_array_equal(x, y)
            for x, y in zip(b.get_monomers(k), a.get_monomers(k)):
                np.testing.assert_array_equal(x, y)


def test_fp64_collide_same_values_from_frame_records_and_recomputed():
    # The FP64 binning stores each solvent particle's collision-frame record
    # (streamed, shifted, wrapped, with its cell key) for the collide that
    # follows. A host write of the solvent between the two phases marks the
    # records stale and the collide recomputes them from the state; writing
    # back the state the binning saw must give the same positions bit for
    # bit either way. Velocities are compared at 1e-13: the FP64 cell sums
    # follow the order the binning's atomics give each cell's particles, so
    # two FP64 runs differ in their last bits even on the same path.
    L, su, h = 10, 1, 0.1
    star, fpos, fvel = H.small_star_system(L=L, shear=0.05, seed=4)
    out = []
    for rewrite in (False, True):
        with H.context_for(star, fpos, fvel, L, 1.0, 0.05, su, rng=capi.RNG_PHILOX,
                           seed=9) as ctx:
            assert ctx.mpc_bin(0, h)
            if rewrite:
                ctx.set_fluid(0, fpos, fvel)
            ctx.mpc_collide()
            ctx.raise_on_device_error()
            p, v = ctx.get_fluid(0)
            mp, mv, _ = ctx.get_monomers(0)
            out.append((p, v, mp, mv))
    (p0, v0, mp0, mv0), (p1, v1, mp1, mv1) = out
    np.testing.assert_array_equal(p0, p1)
    np.testing.assert_array_equal(mp0, mp1)
    H.close64(v0, v1, rtol=1e-13)
    H.close64(mv0, mv1, rtol=1e-13)
