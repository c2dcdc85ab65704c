"""Periodic many-star MD (SMPC_REPLICA_PERIODIC_MD) through the C ABI.

FP64 path: against the oracle's periodic mode (the same Lees-Edwards minimum
image, wrapping and summation order) within 1e-12 of each array's scale, cell
occupancies bit-exact; in the one-star limit against the reference's own
fixtures with the tolerances of the non-periodic replay. Graph-captured
cycles against the same cycles call by call. FP32 path:
stated tolerances against the FP64 oracle.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from starpolymersmd_gb300 import capi, system
from tests import golden_replay as gr
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

L, NC, SU, HSTEP, MD_DT = 12, 3, 5, 0.1, 0.01
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _solution(seed=1, n_stars=4, arms=3, n_arm=5):
    return system.star_solution(n_stars, arms, n_arm, 0.5, 5.0, 1.0, (L, L, L),
                                np.random.default_rng(seed))


def _desc(sol, n_fluid, shear, r_verlet, potential=capi.POT_REF4824, r_cut=1.5, h=HSTEP,
          md_dt=MD_DT):
    return dict(L=(L, L, L), n_fluid=n_fluid, n_mono=sol.n, mol0_size=sol.stars[0].n, kT=1.0,
                shear=shear, h=h, md_dt=md_dt, seed=77, potential=potential, r_cut=r_cut,
                r_verlet=r_verlet, flags=capi.REPLICA_PERIODIC_MD)


def _oracle(sol, fpos, fvel, shear, su, r_verlet, potential=orc.POT_REF4824, r_cut=1.5,
            h=HSTEP, md_dt=MD_DT):
    o = orc.OracleSystem((L, L, L), 1.0, shear, su, len(fpos), sol.n, mol_start=sol.mol_start,
                         md_dt=md_dt, r_cut=r_cut, r_verlet=r_verlet, potential=potential,
                         delrx_dt_scale=1.0 / su, mono_wrap=1)
    o.set_fluid(fpos, fvel)
    o.set_monomers(sol.pos, sol.vel, np.zeros_like(sol.pos), sol.mass, sol.amphi, sol.anchor)
    o.set_bonds(sol.bond_src, sol.bond_dst)
    o.set_periodic_md(h)
    o.init_md()
    o.set_philox(seed=77, counter=0)
    return o


def _context(sol, fpos, fvel, shear, su, r_verlet, precision=capi.FP64, **kw):
    ctx = capi.Context([_desc(sol, len(fpos), shear, r_verlet, **kw)], precision=precision,
                       rng=capi.RNG_PHILOX, step_update=su, mono_bin=capi.MONOBIN_WRAPPED,
                       delrx_mode=capi.DELRX_PHYSICAL)
    if len(fpos):
        ctx.set_fluid(0, fpos, fvel)
    ctx.set_monomers(0, sol.pos, sol.vel, np.zeros_like(sol.pos), sol.mass, sol.amphi,
                     sol.anchor)
    ctx.set_bonds(0, sol.bond_src, sol.bond_dst)
    ctx.set_molecules(0, sol.mol_start)
    ctx.init_md()
    return ctx


def _le_diff(a, b, delrx, shear, va=None, vb=None):
    """a - b for positions in the primary box, modulo the Lees-Edwards images
    (a bead within round-off of a face may sit on either side); with
    velocities, their difference with the image's shear velocity removed."""
    d = np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)
    cy = np.round(d[:, 1] / L)
    d[:, 0] -= cy * delrx
    d[:, 0] -= L * np.round(d[:, 0] / L)
    d[:, 1] -= L * cy
    d[:, 2] -= L * np.round(d[:, 2] / L)
    if va is None:
        return d
    dv = np.asarray(va, dtype=np.float64) - np.asarray(vb, dtype=np.float64)
    dv[:, 0] -= cy * shear * L
    return d, dv


@pytest.mark.parametrize("shear", [0.0, 0.5])
def test_fp64_periodic_md_matches_oracle(shear):
    # four stars straddling the faces, Philox collisions every SU substeps,
    # Verlet skin 0.1 so that the lists are rebuilt several times
    sol = _solution()
    fpos, fvel = system.uniform_fluid((L, L, L), NC, 1.0, np.random.default_rng(11))
    o = _oracle(sol, fpos, fvel, shear, SU, 1.6)
    with _context(sol, fpos, fvel, shear, SU, 1.6) as ctx:
        mp, mv, mf = ctx.get_monomers(0)
        op, ov, of = o.get_monomers()
        assert np.abs(op).max() <= L / 2  # set-up wrapped the stars into the box
        H.close64(mp, op)
        H.close64(mv, ov)
        H.close64(mf, of)
        for t in range(0, 4 * SU + 1):
            o.propagate(False)
            o.mpc_step(t, HSTEP)
            ctx.md_substeps(1)
            ctx.mpc_step(t, HSTEP)
        ctx.raise_on_device_error()
        assert o.error() == 0
        assert ctx.delrx(0) == o.delrx
        tot, fl = ctx.cell_counts(0)
        otot, ofl = o.cell_counts()
        np.testing.assert_array_equal(tot, otot)
        np.testing.assert_array_equal(fl, ofl)
        p, v = ctx.get_fluid(0)
        op, ov = o.get_fluid()
        H.close64(p, op)
        H.close64(v, ov)
        mp, mv, mf = ctx.get_monomers(0)
        op, ov, of = o.get_monomers()
        H.close64(mp, op)
        H.close64(mv, ov)
        H.close64(mf, of)
        assert ctx.verlet_rebuilds(0) >= 3
        H.close64(ctx.temperature(0), o.temperature())


@pytest.mark.parametrize("shear,r_verlet", [(1.0, 1.8), (1.0, 2.0), (0.0, 1.8)])
def test_fp64_periodic_md_long_run_is_the_oracle_to_the_bit(shear, r_verlet):
    # MD only, 400 substeps: one lane per bead and lists in index order give
    # the oracle's sums exactly, so any pair the lists missed (a rebuild
    # criterion that let a pair in range slip through) would show. At shear
    # 1.0 the beads at the y faces move 6 units per time unit with the flow
    # and delrx runs through the box; few rebuilds are due to either.
    sol = _solution(seed=7)
    fpos = np.zeros((0, 3))
    su, md_dt = 1000, 0.002
    h = su * md_dt  # physical delrx advance of md_dt per substep
    kw = dict(h=h, md_dt=md_dt)
    o = _oracle(sol, fpos, fpos, shear, su, r_verlet, **kw)
    with _context(sol, fpos, fpos, shear, su, r_verlet, **kw) as ctx:
        n = 400
        for t in range(1, n + 1):
            o.propagate(False)
            o.mpc_step(t, h)  # delrx advance only
        ctx.md_substeps(n)
        ctx.raise_on_device_error()
        for x, y in zip(ctx.get_monomers(0), o.get_monomers()):
            np.testing.assert_array_equal(x, y)
        rebuilds = ctx.verlet_rebuilds(0)
        assert 2 <= rebuilds < 100


def test_fp64_periodic_epot_matches_oracle():
    sol = _solution(seed=4)
    fpos = np.zeros((0, 3))
    o = _oracle(sol, fpos, fpos, 0.2, 50, 2.0)
    with _context(sol, fpos, fpos, 0.2, 50, 2.0) as ctx:
        for t in range(1, 13):
            o.propagate(True)
            o.mpc_step(t, HSTEP)  # delrx advance only (t % 50 != 0)
        ctx.md_substeps(12, calc_epot=True)
        ctx.raise_on_device_error()
        H.close64(ctx.epot(0), o.epot())
        for x, y in zip(ctx.get_monomers(0), o.get_monomers()):
            H.close64(x, y)


def test_fp64_periodic_graph_cycles_match_stepwise():
    sol = _solution(seed=2)
    fpos, fvel = system.uniform_fluid((L, L, L), NC, 1.0, np.random.default_rng(12))
    with _context(sol, fpos, fvel, 0.3, SU, 1.8) as a, \
            _context(sol, fpos, fvel, 0.3, SU, 1.8) as b:
        for t in range(1, 3 * SU + 1):
            a.md_substeps(1)
            a.mpc_step(t, HSTEP)
        b.cycles(3)
        b.synchronize()
        a.raise_on_device_error()
        b.raise_on_device_error()
        assert a.delrx(0) == b.delrx(0)
        # as for one star: the FP64 per-cell sums run in the order the binning
        # atomics ranked each cell's particles, so the two runs agree to
        # round-off; the lists are rebuilt on the same substeps
        for x, y in zip(b.get_fluid(0), a.get_fluid(0)):
            H.close64(x, y)
        for x, y in zip(b.get_monomers(0), a.get_monomers(0)):
            H.close64(x, y)
        assert a.verlet_rebuilds(0) == b.verlet_rebuilds(0)


@pytest.mark.parametrize("pmd_variant", [0, 1, 2, 3])
def test_fp32_periodic_md_tracks_fp64_oracle(pmd_variant):
    # MD only (no collision in 40 substeps), 12-6 preset with LJ attraction to
    # 2.5 and skin 0.3, shear 0.5: FP32 against the FP64 oracle, with every
    # launch shape of the periodic MD (4, 8 or 16 lanes per bead)
    sol = _solution(seed=3, n_stars=6, arms=4, n_arm=6)
    su = 50
    fpos = np.zeros((0, 3))
    kw = dict(potential=capi.POT_LJ126, r_cut=2.5)
    o = _oracle(sol, fpos, fpos, 0.5, su, 2.8, potential=orc.POT_LJ126, r_cut=2.5)
    with _context(sol, fpos, fpos, 0.5, su, 2.8, precision=capi.FP32, **kw) as ctx:
        ctx.set_pmd_variant(pmd_variant)
        assert ctx.get_pmd_variant() == pmd_variant
        n = 40
        for t in range(1, n + 1):
            o.propagate(False)
            o.mpc_step(t, HSTEP)
        ctx.md_substeps(n)
        ctx.raise_on_device_error()
        assert o.error() == 0
        mp, mv, mf = ctx.get_monomers(0)
        op, ov, of = o.get_monomers()
        dp, dv = _le_diff(mp, op, o.delrx, 0.5, mv, ov)
        assert np.abs(dp).max() < 1e-4
        assert np.abs(dv).max() < 2e-3 * np.abs(ov).max()
        np.testing.assert_allclose(mf, of, atol=2e-3 * np.abs(of).max())


@pytest.mark.parametrize("name", ["star_mpc_L12", "md_saw_L16"])
def test_periodic_md_of_one_star_replays_reference_fixture(name):
    # one star away from the faces: the periodic form reduces to the
    # reference's MD (its own fixtures, injected draws), up to the order of
    # the force sums
    fx = gr.load(os.path.join(GOLDEN, name + ".npz"))
    coll = gr.collision_index(fx)
    with H.fixture_context(fx, periodic=True) as ctx:
        _, _, f0 = ctx.get_monomers(0)
        H.close64(f0, fx["mono_force0"])
        for t in range(int(fx["n_loop"])):
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
                    p, v = ctx.get_fluid(0)
                    H.close64(p, fx["fluid_pos"][k])
                    H.close64(v, fx["fluid_vel"][k])
                    if "observables" in fx:
                        H.close64(ctx.molecule_observables_all()[0], fx["observables"][k])
                else:
                    ctx.mpc_step(t, float(fx["h"]))
            p, v, f = ctx.get_monomers(0)
            H.close64(p, fx["mono_pos"][t])
            H.close64(v, fx["mono_vel"][t])
            H.close64(f, fx["mono_force"][t], rtol=1e-11)
        ctx.raise_on_device_error()


def _numpy_unwrap(pos, vel, src, dst, mol_start, delrx, shear):
    """Molecules made whole: bead i next to its lowest-indexed bonded partner
    of the same molecule (else the molecule's first bead), at the
    Lees-Edwards minimum image, v_x shifted by the image's shear velocity."""
    n = len(pos)
    nb = [[] for _ in range(n)]
    for s, d in zip(src, dst):
        nb[s].append(d)
        nb[d].append(s)
    up, uv = pos.copy(), vel.copy()
    for a, b in zip(mol_start[:-1], mol_start[1:]):
        for i in range(a + 1, b):
            cands = [j for j in nb[i] if a <= j < i]
            p = min(cands) if cands else a
            d = pos[i] - pos[p]
            cy = np.round(d[1] / L)
            d[0] -= L * np.round(d[0] / L)
            d[0] -= cy * delrx
            d[0] -= L * np.round(d[0] / L)
            d[1] -= L * cy
            d[2] -= L * np.round(d[2] / L)
            up[i] = up[p] + d
            uv[i, 0] = vel[i, 0] + np.round((up[i, 1] - pos[i, 1]) / L) * shear * L
    return up, uv


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_periodic_observables_use_whole_molecules(precision):
    from tests.test_gpu_parity import _numpy_observables
    sol = _solution(seed=5)
    fpos, fvel = system.uniform_fluid((L, L, L), NC, 1.0, np.random.default_rng(13))
    shear = 0.3
    with _context(sol, fpos, fvel, shear, SU, 1.8, precision=precision) as ctx:
        for t in range(1, 2 * SU + 1):
            ctx.md_substeps(1)
            ctx.mpc_step(t, HSTEP)
        ctx.raise_on_device_error()
        pos, vel, _ = ctx.get_monomers(0)
        # the set-up wrap split at least one star across a face
        ms = sol.mol_start
        assert any(np.ptp(pos[a:b], axis=0).max() > L / 2 for a, b in zip(ms[:-1], ms[1:]))
        up, uv = _numpy_unwrap(pos, vel, sol.bond_src, sol.bond_dst, ms, ctx.delrx(0), shear)
        want = _numpy_observables(up, uv, sol.mass, ms)
        got = ctx.molecule_observables_all()[0]
        tol = 1e-9 if precision == capi.FP64 else 1e-4
        np.testing.assert_allclose(got, want, rtol=tol, atol=tol * np.abs(want).max())
        # whole stars stay compact: no bond of the unwrapped copy spans a face
        d = up[sol.bond_dst] - up[sol.bond_src]
        assert np.sqrt((d * d).sum(axis=1)).max() < 4.5


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_state_set_from_outside_rebuilds_the_lists(precision):
    # The periodic rebuild criterion integrates the peculiar displacement, so
    # it cannot see positions placed by smpc_set_monomer_state_all: the upload
    # requests a list rebuild at the next substep. The stored forces stay those
    # of the old positions (velocity Verlet carries them between calls), so a
    # rewind to an earlier configuration calls smpc_init_md, and must then
    # replay the same trajectory bit for bit.
    sol = _solution(seed=3)
    empty = np.zeros((0, 3))
    # 12-6 preset (capped FENE): stable without a thermostat
    with _context(sol, empty, empty, 0.2, 1000, 2.8, precision=precision,
                  potential=capi.POT_LJ126, r_cut=2.5, md_dt=0.005) as ctx:
        n = sol.n
        state = lambda: (np.zeros((n, 3)), np.zeros((n, 3)))
        ctx.md_substeps(10)
        p0, v0 = state()
        ctx.get_monomer_state_all(p0, v0)
        ctx.md_substeps(400)
        p1, v1 = state()
        ctx.get_monomer_state_all(p1, v1)
        assert np.all(np.isfinite(p1)) and np.all(np.isfinite(v1))
        assert np.abs(H.wrapped_diff(p1, p0, (L, L, L))).max() > 0.3  # the beads did move
        # the upload alone: a rebuild at the next substep
        r0 = ctx.verlet_rebuilds(0)
        ctx.set_monomer_state_all(p1, v1)
        ctx.md_substeps(1)
        assert ctx.verlet_rebuilds(0) == r0 + 1
        # rewind: positions, velocities and (init_md) their forces
        ctx.set_monomer_state_all(p0, v0)
        ctx.init_md()
        ctx.md_substeps(400)
        p2, v2 = state()
        ctx.get_monomer_state_all(p2, v2)
        ctx.raise_on_device_error()
        np.testing.assert_array_equal(p2, p1)
        np.testing.assert_array_equal(v2, v1)


@pytest.mark.parametrize("interleave", [False, True])
def test_unwrap_of_long_and_interleaved_molecules(interleave):
    # Molecules made whole by the device against numpy: stars of 8 x 40 beads
    # span several 256-bead chunks (the block scan carries segments across
    # warps and chunks); with the arms numbered round-robin every partner sits
    # 8 beads back inside the chunk, which takes the one-by-one walk.
    from tests.test_gpu_parity import _numpy_observables
    rng = np.random.default_rng(21)
    Lb = 40
    sol = system.star_solution(3, 8, 40, 0.5, 5.0, 1.0, (Lb, Lb, Lb), rng, bond=0.97)
    pos, vel, mass = sol.pos.copy(), sol.vel.copy(), np.asarray(sol.mass).copy()
    amphi, anchor = np.asarray(sol.amphi).copy(), np.asarray(sol.anchor).copy()
    src, dst = np.asarray(sol.bond_src).copy(), np.asarray(sol.bond_dst).copy()
    ms = list(sol.mol_start)
    if interleave:
        perm = np.arange(len(pos))  # new index -> old index
        for a, b in zip(ms[:-1], ms[1:]):
            arms, n_arm = 8, 40
            old = [a] + [a + 1 + arm * n_arm + k for k in range(n_arm) for arm in range(arms)]
            perm[a:b] = old
        inv = np.empty_like(perm)
        inv[perm] = np.arange(len(perm))
        pos, vel, mass, amphi, anchor = pos[perm], vel[perm], mass[perm], amphi[perm], anchor[perm]
        src, dst = inv[src], inv[dst]
    desc = dict(L=(Lb, Lb, Lb), n_fluid=0, n_mono=len(pos), mol0_size=ms[1], kT=1.0, shear=0.2,
                h=0.1, md_dt=0.005, seed=5, potential=capi.POT_LJ126, r_cut=2.5, r_verlet=2.8,
                flags=capi.REPLICA_PERIODIC_MD)
    with capi.Context([desc], precision=capi.FP64, rng=capi.RNG_PHILOX, step_update=10,
                      mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL) as ctx:
        ctx.set_monomers(0, pos, vel, np.zeros_like(pos), mass, amphi, anchor)
        ctx.set_bonds(0, src, dst)
        ctx.set_molecules(0, ms)
        ctx.init_md()
        ctx.md_substeps(20)
        ctx.raise_on_device_error()
        p, v, _ = ctx.get_monomers(0)
        up, uv = _numpy_unwrap_L(p, v, src, dst, ms, ctx.delrx(0), 0.2, Lb)
        want = _numpy_observables(up, uv, mass, ms)
        got = ctx.molecule_observables_all()[0]
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * np.abs(want).max())


def _numpy_unwrap_L(pos, vel, src, dst, mol_start, delrx, shear, Lb):
    n = len(pos)
    nb = [[] for _ in range(n)]
    for s, d in zip(src, dst):
        nb[s].append(d)
        nb[d].append(s)
    up, uv = pos.copy(), vel.copy()
    for a, b in zip(mol_start[:-1], mol_start[1:]):
        for i in range(a + 1, b):
            cands = [j for j in nb[i] if a <= j < i]
            p = min(cands) if cands else a
            d = pos[i] - pos[p]
            cy = np.round(d[1] / Lb)
            d[0] -= Lb * np.round(d[0] / Lb)
            d[0] -= cy * delrx
            d[0] -= Lb * np.round(d[0] / Lb)
            d[1] -= Lb * cy
            d[2] -= Lb * np.round(d[2] / Lb)
            up[i] = up[p] + d
            uv[i, 0] = vel[i, 0] + np.round((up[i, 1] - pos[i, 1]) / Lb) * shear * Lb
    return up, uv


def test_autotune_covers_the_periodic_md_shapes():
    # a context with a periodic box gets the periodic-MD category, keeps its
    # choice, and the trial cycles leave the state where it was
    sol = _solution(seed=4, n_stars=4, arms=4, n_arm=6)
    rng = np.random.default_rng(12)
    fpos = (rng.random((3 * L ** 3, 3)) - 0.5) * L
    fvel = rng.normal(0.0, 1.0, fpos.shape)
    kw = dict(potential=capi.POT_LJ126, r_cut=2.5)
    with _context(sol, fpos, fvel, 0.2, 10, 2.8, precision=capi.FP32, **kw) as a, \
            _context(sol, fpos, fvel, 0.2, 10, 2.8, precision=capi.FP32, **kw) as b:
        a.cycles(2)
        b.cycles(2)
        report = a.autotune(1)
        assert {"fluid_bin", "collide", "md_substeps", "pmd"} <= set(report)
        assert a.get_pmd_variant() == report["pmd"]["index"]
        b.set_variants(*a.get_variants())
        b.set_pmd_variant(a.get_pmd_variant())
        a.cycles(2)
        b.cycles(2)
        a.raise_on_device_error()
        b.raise_on_device_error()
        for x, y in zip(a.get_fluid(0) + a.get_monomers(0), b.get_fluid(0) + b.get_monomers(0)):
            np.testing.assert_array_equal(x, y)
