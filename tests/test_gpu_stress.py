"""Pressure tensor on the device (smpc_pressure_tensor_all) against a numpy
restatement of its definition on the same state: kinetic part with the
peculiar velocity v - shear y e_x over solvent and monomers, monomer pair and
FENE virial over all pairs (Lees-Edwards minimum image in periodic boxes)."""
import numpy as np
import pytest

from starpolymersmd_gb300 import capi, system
from tests import gpu_helpers as H
from tests.test_gpu_periodic import _context as periodic_context, _solution

pytestmark = pytest.mark.gpu


def _pair_fa(pot, bb, r2, lam):
    fa = np.zeros_like(r2)
    if pot == capi.POT_REF4824:
        rm2 = 1.0 / r2
        rm24 = rm2 ** 12
        f = 192.0 * rm2 * rm24 * (rm24 - 0.5)
        fa = np.where(r2 < 1.0594631, f, np.where(bb & (r2 < 2.25), lam * f, 0.0))
    else:
        rm2 = 1.0 / r2
        rm6 = rm2 ** 3
        f = 48.0 * rm2 * rm6 * (rm6 - 0.5)
        fa = np.where(r2 < 2.0 ** (1.0 / 3.0), f, np.where(bb & (r2 < 6.25), lam * f, 0.0))
    return fa


def _min_image(d, L, delrx):
    d = d.copy()
    cy = np.round(d[..., 1] / L)
    d[..., 0] -= L * np.round(d[..., 0] / L)
    d[..., 0] -= cy * delrx
    d[..., 0] -= L * np.round(d[..., 0] / L)
    d[..., 1] -= L * cy
    d[..., 2] -= L * np.round(d[..., 2] / L)
    return d


def _tensor(a, b, w):
    return np.array([np.sum(w * a[:, 0] * b[:, 0]), np.sum(w * a[:, 1] * b[:, 1]),
                     np.sum(w * a[:, 2] * b[:, 2]), np.sum(w * a[:, 0] * b[:, 1]),
                     np.sum(w * a[:, 0] * b[:, 2]), np.sum(w * a[:, 1] * b[:, 2])])


def _numpy_pressure(fpos, fvel, mpos, mvel, mass, amphi, anchor, src, dst, L, shear, delrx,
                    periodic, pot, lam):
    V = float(L) ** 3
    u = fvel.copy()
    u[:, 0] -= shear * fpos[:, 1]
    kin = _tensor(u, u, 1.0)
    um = mvel.copy()
    um[:, 0] -= shear * mpos[:, 1]
    kin += _tensor(um, um, mass)
    n = len(mpos)
    i, j = np.triu_indices(n, 1)
    d = mpos[j] - mpos[i]
    if periodic:
        d = _min_image(d, L, delrx)
    r2 = (d * d).sum(axis=1)
    fa = _pair_fa(pot, (amphi[i] == 1) & (amphi[j] == 1), r2, lam)
    vir = _tensor(d, d, fa)
    db = mpos[dst] - mpos[src]
    if periodic:
        db = _min_image(db, L, delrx)
    rb = (db * db).sum(axis=1)
    R0 = np.where(anchor[src] == 1, 20.25, 2.25)
    if pot != capi.POT_REF4824:
        rb = np.minimum(rb, 0.98 * R0)
    vir += _tensor(db, db, -30.0 / (1.0 - rb / R0))
    return kin / V, vir / V


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_pressure_tensor_of_a_periodic_solution(precision):
    L = 12
    sol = _solution(seed=9)
    fpos, fvel = system.uniform_fluid((L, L, L), 3, 1.0, np.random.default_rng(3))
    with periodic_context(sol, fpos, fvel, 0.4, 5, 2.8, precision=precision,
                          potential=capi.POT_LJ126, r_cut=2.5) as ctx:
        for t in range(1, 11):
            ctx.md_substeps(1)
            ctx.mpc_step(t, 0.1)
        ctx.raise_on_device_error()
        kin, vir = ctx.pressure_tensor_all()
        fp, fv = ctx.get_fluid(0)
        mp, mv, _ = ctx.get_monomers(0)
        wk, wv = _numpy_pressure(fp, fv, mp, mv, sol.mass, sol.amphi, sol.anchor, sol.bond_src,
                                 sol.bond_dst, L, 0.4, ctx.delrx(0), True, capi.POT_LJ126, 1.0)
        tol = 1e-10 if precision == capi.FP64 else 2e-5
        np.testing.assert_allclose(kin[0], wk, rtol=tol, atol=tol * np.abs(wk).max())
        np.testing.assert_allclose(vir[0], wv, rtol=tol, atol=tol * np.abs(wv).max())


def test_pressure_tensor_of_one_star():
    L = 10
    star, fpos, fvel = H.small_star_system(L=L, shear=0.1, seed=4)
    with H.context_for(star, fpos, fvel, L, 1.0, 0.1, 5, rng=capi.RNG_PHILOX, seed=2) as ctx:
        for t in range(1, 6):
            ctx.md_substeps(1)
            ctx.mpc_step(t, 0.1)
        ctx.raise_on_device_error()
        kin, vir = ctx.pressure_tensor_all()
        fp, fv = ctx.get_fluid(0)
        mp, mv, _ = ctx.get_monomers(0)
        wk, wv = _numpy_pressure(fp, fv, mp, mv, np.full(star.n, star.mass), star.amphi,
                                 star.anchor, star.bond_src, star.bond_dst, L, 0.1, 0.0, False,
                                 capi.POT_REF4824, 1.0)
        np.testing.assert_allclose(kin[0], wk, rtol=1e-10, atol=1e-10 * np.abs(wk).max())
        np.testing.assert_allclose(vir[0], wv, rtol=1e-10, atol=1e-10 * np.abs(wv).max())
        # the solvent alone, at rest on average in the flow frame: kT on the diagonal
        assert np.all(np.abs(kin[0][:3] * L ** 3 / len(fp) - 1.0) < 0.3)


def test_precision_report_runs_both_paths():
    # the FP32-versus-FP64 report on a small workload: both runs sample, the
    # momentum along y and z is conserved, the kinetic temperature is near kT
    from starpolymersmd_gb300 import precision_report as P
    r = P.report("single_star_20", cycles=6, every=2)
    assert set(r["momentum_yz_drift_per_particle"]) == {"fp32", "fp64"}
    assert r["momentum_yz_drift_per_particle"]["fp64"] < 1e-12
    assert r["momentum_yz_drift_per_particle"]["fp32"] < 1e-6
    for name in ("fp32", "fp64"):
        assert abs(r["temperature_kinetic"][name] - 1.0) < 0.1  # the flow is not yet steady
    assert len(r["gyration"]["fp32"]) == 9
