"""Parity at the benchmark configurations' sizes, through the C ABI.

FP64 path against the C oracle at 1e-12 (relative to each array's scale),
cell occupancies and every particle's cell bit-exact:
  * config 1 exactly: one star f = 6, N_arm = 20 (121 beads, mass 5) in a
    20^3 box at rho = 10, shear 0.05, 10 MD substeps per collision, the
    reference's 48-24 pair preset, reference delrx and monomer binning, driven
    call by call like star-polymers.cpp:530-534 and as captured graph cycles;
  * the config-2 star (f = 10, N_arm = 40, 401 beads) in a 30^3 box at the
    sweep's strongest shear 0.2;
  * four replicas of the 256-replica benchmark table with the largest stars
    (721 beads in L = 29; 661, 595 and 571 beads in L = 36, 36, 40) in one
    batched context with the benchmark's production options, against one
    oracle per replica.
FP32 path against the oracle run on the FP32 path's own 23-bit uniforms,
one cycle at a time from the FP32 state: every particle must agree to FP32
accuracy except those in the few cells where a particle within FP32 rounding
of a cell face was binned differently (counted and bounded).
A cell of several thousand particles (beyond the collide tile's staging
capacity and the int32 split accumulators) is replayed on injected draws.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from starpolymersmd_gb300 import capi, system, workloads as W
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

H_MPC = 0.1
N_SUB = 10
BIG_SEEDS = (139, 84, 11, 179)  # batched_replica_table(256): the largest stars


def _compare_fp64(ctx, o, rep=0, mono=True):
    tot, fl = ctx.cell_counts(rep)
    otot, ofl = o.cell_counts()
    np.testing.assert_array_equal(tot, otot)
    np.testing.assert_array_equal(fl, ofl)
    fc, mc = ctx.cell_members(rep)
    ofc, omc = o.cell_members()
    np.testing.assert_array_equal(fc, ofc)
    np.testing.assert_array_equal(mc, omc)
    p, v = ctx.get_fluid(rep)
    op, ov = o.get_fluid()
    H.close64(p, op)
    H.close64(v, ov)
    if mono:
        mp, mv, mf = ctx.get_monomers(rep)
        omp, omv, omf = o.get_monomers()
        H.close64(mp, omp)
        H.close64(mv, omv)
        H.close64(mf, omf, rtol=1e-11)
    H.close64(ctx.temperature(rep), o.temperature())
    assert ctx.delrx(rep) == o.delrx


def _config1_system(seed=1):
    # positions uniform, Maxwell-Boltzmann velocities, self-avoiding star from
    # the box centre (config 1's initialisation), kept inside the reference's
    # box-bounded Verlet grid
    rng = np.random.default_rng(seed)
    for _ in range(200):
        star = system.make_star(6, 20, 0.5, 5.0, 1.0, rng, bond=1.01, outward_bias=0.0)
        if np.abs(star.pos).max() < 20 / 2 - 1.5:
            break
    fpos, fvel = system.uniform_fluid((20, 20, 20), 10, 1.0, rng)
    return star, fpos, fvel


def test_fp64_config1_stepwise_matches_oracle():
    L, shear = 20, 0.05
    star, fpos, fvel = _config1_system()
    assert star.n == 121 and len(fpos) == 80000
    o = H.oracle_for(star, fpos, fvel, L, 1.0, shear, N_SUB)
    o.set_philox(seed=1, counter=0)
    with H.context_for(star, fpos, fvel, L, 1.0, shear, N_SUB, rng=capi.RNG_PHILOX,
                       seed=1) as ctx:
        for t in range(0, 3 * N_SUB + 1):
            o.propagate(False)
            o.mpc_step(t, H_MPC)
            ctx.md_substeps(1)
            ctx.mpc_step(t, H_MPC)
            if t % N_SUB == 0:
                ctx.raise_on_device_error()
                assert o.error() == 0
                _compare_fp64(ctx, o)


def test_fp64_config1_graph_cycles_match_oracle():
    L, shear = 20, 0.05
    star, fpos, fvel = _config1_system(seed=2)
    o = H.oracle_for(star, fpos, fvel, L, 1.0, shear, N_SUB)
    o.set_philox(seed=3, counter=0)
    with H.context_for(star, fpos, fvel, L, 1.0, shear, N_SUB, rng=capi.RNG_PHILOX,
                       seed=3) as ctx:
        for k in range(3):
            ctx.cycles(1)
            ctx.synchronize()
            ctx.raise_on_device_error()
            o.run(1 + N_SUB * k, N_SUB, H_MPC, True)  # collision at the 10th call
            assert o.error() == 0
            _compare_fp64(ctx, o)


def test_fp64_config2_star_matches_oracle():
    L, shear = 30, 0.2
    star, fpos, fvel = H.small_star_system(L=L, arms=10, n_arm=40, frac=0.5, shear=shear,
                                           seed=3)
    assert star.n == 401
    o = H.oracle_for(star, fpos, fvel, L, 1.0, shear, N_SUB)
    o.set_philox(seed=7, counter=0)
    with H.context_for(star, fpos, fvel, L, 1.0, shear, N_SUB, rng=capi.RNG_PHILOX,
                       seed=7) as ctx:
        for k in range(2):
            ctx.cycles(1)
            ctx.synchronize()
            ctx.raise_on_device_error()
            o.run(1 + N_SUB * k, N_SUB, H_MPC, True)
            assert o.error() == 0
            _compare_fp64(ctx, o)


def _big_replicas(precision):
    """The four largest-star replicas of the benchmark table, built like the
    benchmark (stars, device-drawn solvent, production options), and one
    oracle per replica loaded with the same state."""
    table = {s.seed: s for s in system.batched_replica_table(256)}
    specs = [table[s] for s in BIG_SEEDS]
    built = W.build(specs, precision=precision)
    oracles = []
    for k, (s, st) in enumerate(zip(specs, built.stars)):
        fp, fv = built.ctx.get_fluid(k)
        mp, mv, mf = built.ctx.get_monomers(k)
        o = orc.OracleSystem((s.L,) * 3, s.kT, s.shear, N_SUB, len(fp), st.n,
                             mol_start=[0, st.n], lambda_=1.0, md_dt=W.MD_DT,
                             r_cut=W.R_CUT_LJ, r_verlet=W.R_CUT_LJ + W.SKIN,
                             potential=orc.POT_LJ126, delrx_dt_scale=1.0 / N_SUB, mono_wrap=1)
        o.set_fluid(fp, fv)
        o.set_monomers(mp, mv, mf, np.full(st.n, st.mass), st.amphi, st.anchor)
        o.set_bonds(st.bond_src, st.bond_dst)
        o.init_md()
        o.set_philox(s.seed, 0)
        oracles.append(o)
    return built, specs, oracles


def test_fp64_largest_batched_replicas_match_oracles():
    built, specs, oracles = _big_replicas(capi.FP64)
    assert max(st.n for st in built.stars) == 721
    with built.ctx as ctx:
        for k, o in enumerate(oracles):  # the same start: forces from init_md
            _, _, mf = ctx.get_monomers(k)
            H.close64(mf, o.get_monomers()[2], rtol=1e-11)
        for c in range(2):
            ctx.cycles(1)
            ctx.synchronize()
            ctx.raise_on_device_error()
            for k, o in enumerate(oracles):
                o.run(1 + N_SUB * c, N_SUB, H_MPC, True)
                assert o.error() == 0
                _compare_fp64(ctx, o, rep=k)


# ----------------------------------------------------------------- FP32

def test_fp32_config1_tracks_f32_uniform_oracle():
    L, shear = 20, 0.05
    star, fpos, fvel = _config1_system(seed=4)
    kw = dict(rng=capi.RNG_PHILOX, seed=11, precision=capi.FP32, potential=capi.POT_LJ126,
              r_cut=W.R_CUT_LJ, r_verlet=W.R_CUT_LJ + W.SKIN, mono_bin=capi.MONOBIN_WRAPPED,
              strict=0, delrx_mode=capi.DELRX_PHYSICAL)
    o = orc.OracleSystem((L,) * 3, 1.0, shear, N_SUB, len(fpos), star.n, mol_start=[0, star.n],
                         lambda_=1.0, md_dt=0.01, r_cut=W.R_CUT_LJ, r_verlet=W.R_CUT_LJ + W.SKIN,
                         potential=orc.POT_LJ126, delrx_dt_scale=1.0 / N_SUB, mono_wrap=1)
    o.set_monomers(star.pos, star.vel, np.zeros_like(star.pos), np.full(star.n, star.mass),
                   star.amphi, star.anchor)
    o.set_bonds(star.bond_src, star.bond_dst)
    o.set_fluid(fpos, fvel)
    o.init_md()
    o.set_philox(11, 0)
    o.set_f32_uniforms(True)
    flips = 0
    with H.context_for(star, fpos, fvel, L, 1.0, shear, N_SUB, **kw) as ctx:
        for c in range(5):
            H.resync_oracle(ctx, o, 0)
            ctx.cycles(1)
            ctx.synchronize()
            ctx.raise_on_device_error()
            o.run(1 + N_SUB * c, N_SUB, H_MPC, True)
            assert o.error() == 0
            flips += H.fp32_cycle_check(ctx, o, 0, L)
    assert flips <= 20


def test_fp32_largest_batched_replicas_track_f32_uniform_oracles():
    built, specs, oracles = _big_replicas(capi.FP32)
    for o in oracles:
        o.set_f32_uniforms(True)
    with built.ctx as ctx:
        for c in range(2):
            for k, o in enumerate(oracles):
                H.resync_oracle(ctx, o, k)
            ctx.cycles(1)
            ctx.synchronize()
            ctx.raise_on_device_error()
            for k, (o, s) in enumerate(zip(oracles, specs)):
                o.run(1 + N_SUB * c, N_SUB, H_MPC, True)
                assert o.error() == 0
                H.fp32_cycle_check(ctx, o, k, s.L)


# ------------------------------------------------------ a very full cell

@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_cell_of_thousands_matches_oracle(precision):
    # 3000 solvent particles at rest near the centre of one cell, inside a
    # uniform solvent: with no grid shift the cell keeps them all, so one
    # collision sees a cell of ~3010 particles (beyond the 704-particle tile
    # staging and the 1024-particle split accumulators of the FP32 kernel)
    L = 8
    rng = np.random.default_rng(21)
    fpos, fvel = system.uniform_fluid((L,) * 3, 10, 1.0, rng)
    k = 3000
    cpos = np.full((k, 3), 0.5) + (rng.random((k, 3)) - 0.5) * 0.1
    fpos = np.concatenate([fpos, cpos])
    fvel = np.concatenate([fvel, np.zeros((k, 3))])
    fvel[-k:, 0] = rng.normal(0.0, 1e-3, k)  # not all equal: the rotation acts
    n_cell = L ** 3
    shift = np.zeros(3)
    gamma = rng.gamma(1.5 * 3009, 1.0, n_cell)
    uphi, uth = rng.random(n_cell), rng.random(n_cell)
    rep = dict(L=(L,) * 3, n_fluid=len(fpos), kT=1.0, shear=0.0, h=H_MPC, seed=1)
    o = orc.OracleSystem((L,) * 3, 1.0, 0.0, 1, len(fpos))
    o.set_fluid(fpos, fvel)
    o.set_inject(shift, gamma, uphi, uth)
    o.mpc_step(0, H_MPC)
    assert o.error() == 0
    tot, _ = o.cell_counts()
    assert tot.max() > 3000
    with capi.Context([rep], precision=precision, rng=capi.RNG_INJECT, step_update=1) as ctx:
        ctx.set_fluid(0, fpos, fvel)
        ctx.mpc_step(0, H_MPC, shift, gamma, uphi, uth)
        ctx.raise_on_device_error()
        gtot, _ = ctx.cell_counts(0)
        np.testing.assert_array_equal(gtot, tot)
        p, v = ctx.get_fluid(0)
        op, ov = o.get_fluid()
        if precision == capi.FP64:
            H.close64(p, op)
            H.close64(v, ov)
        else:
            assert np.abs(H.wrapped_diff(p, op, (L,) * 3)).max() < 1e-6 * L
            assert np.abs(v - ov).max() < H.FP32_VEL_RTOL * np.abs(ov).max()
