"""Solvent initialisation on the device (smpc_init_solvent).

MPC::initialize (MPC.cpp:34-55) places the solvent uniformly in the box and
draws velocities, then removes their mean. smpc_init_solvent does the same
with counter-based draws (uniform velocities with SMPC_INIT_REFERENCE_VELOCITIES,
Maxwell-Boltzmann at kT otherwise) and can add the steady Lees-Edwards flow
(SMPC_INIT_SHEAR_PROFILE). Checked statistically on 138,240 particles:
occupancy of the cells (chi-squared against the uniform multinomial), zero
total momentum, the temperature, the velocity distribution and the profile.
"""
import numpy as np
import pytest

from starpolymersmd_gb300 import capi

pytestmark = pytest.mark.gpu

L, NC = 24, 10
N = NC * L ** 3


def _draw(precision, flags=(), kT=1.0, shear=0.0, seed=7):
    rep = dict(L=(L,) * 3, n_fluid=N, kT=kT, shear=shear, h=0.1, seed=1)
    with capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX, step_update=1) as ctx:
        ctx.init_solvent(0, seed=seed, reference_velocities="ref" in flags,
                         shear_profile="shear" in flags)
        return ctx.get_fluid(0)


def _momentum_tol(precision):
    return 1e-12 if precision == capi.FP64 else 1e-6


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_positions_uniform_in_the_box(precision):
    pos, _ = _draw(precision)
    assert pos.shape == (N, 3)
    assert np.all(pos >= -L / 2) and np.all(pos < L / 2)
    cell = np.floor(pos + L / 2).astype(np.int64)
    idx = cell[:, 0] + L * (cell[:, 1] + L * cell[:, 2])
    counts = np.bincount(idx, minlength=L ** 3)
    chi2 = float(((counts - NC) ** 2).sum() / NC)
    dof = L ** 3 - 1
    assert abs(chi2 - dof) < 6.0 * np.sqrt(2.0 * dof), chi2
    # every axis uniform on its own too
    for d in range(3):
        h = np.bincount(cell[:, d], minlength=L)
        c2 = float(((h - N / L) ** 2).sum() / (N / L))
        assert c2 < (L - 1) + 6.0 * np.sqrt(2.0 * (L - 1)), (d, c2)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("kT", [1.0, 0.5])
def test_maxwell_boltzmann_velocities(precision, kT):
    _, vel = _draw(precision, kT=kT)
    # the mean is removed (MPC.cpp:42-48): zero total momentum
    assert np.abs(vel.mean(axis=0)).max() < _momentum_tol(precision) * np.sqrt(kT)
    # equipartition with one degree of freedom per axis removed by the mean
    T = float((vel ** 2).sum() / (3.0 * (N - 1)))
    assert abs(T / kT - 1.0) < 6.0 * np.sqrt(2.0 / (3.0 * N)), T
    # Gaussian components: fraction within one standard deviation, kurtosis
    s = vel / np.sqrt(kT)
    p1 = float((np.abs(s) < 1.0).mean())
    assert abs(p1 - 0.682689492) < 6.0 * np.sqrt(0.68 * 0.32 / (3 * N)), p1
    kurt = float((s ** 4).mean() / (s ** 2).mean() ** 2)
    assert abs(kurt - 3.0) < 6.0 * np.sqrt(24.0 / (3 * N)), kurt
    # components uncorrelated
    c = np.corrcoef(vel.T)
    assert np.abs(c - np.eye(3)).max() < 6.0 / np.sqrt(N)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_reference_velocities(precision):
    # Rand::real_uniform() - 0.5 per component, minus the mean (MPC.cpp:40-47)
    _, vel = _draw(precision, flags=("ref",))
    assert np.abs(vel.mean(axis=0)).max() < _momentum_tol(precision)
    assert vel.min() > -0.5 - 1e-2 and vel.max() < 0.5 + 1e-2
    var = vel.var(axis=0)
    assert np.abs(var - 1.0 / 12.0).max() < 6.0 * np.sqrt(1.0 / 180.0 / N)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_shear_profile(precision):
    shear = 0.2
    pos, vel = _draw(precision, flags=("shear",), shear=shear)
    u = vel.copy()
    u[:, 0] -= shear * pos[:, 1]
    # thermal part: zero mean, kT
    assert np.abs(u.mean(axis=0)).max() < 10 * _momentum_tol(precision)
    T = float((u ** 2).sum() / (3.0 * (N - 1)))
    assert abs(T - 1.0) < 6.0 * np.sqrt(2.0 / (3.0 * N))
    # v_x = shear * y: least-squares slope within its standard error
    y = pos[:, 1]
    slope = float(((y - y.mean()) * (vel[:, 0] - vel[:, 0].mean())).sum() / ((y - y.mean()) ** 2).sum())
    se = 1.0 / np.sqrt(((y - y.mean()) ** 2).sum())
    assert abs(slope - shear) < 6.0 * se, (slope, se)
    np.testing.assert_allclose(vel[:, 1:], u[:, 1:])


def test_seeds():
    a = _draw(capi.FP64, seed=3)
    b = _draw(capi.FP64, seed=3)
    c = _draw(capi.FP64, seed=4)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert np.abs(a[0] - c[0]).max() > 1.0
    # the FP32 state is the FP64 state rounded to float (same draws)
    f = _draw(capi.FP32, seed=3)
    np.testing.assert_allclose(f[0], a[0], rtol=0, atol=4e-6 * L)
    np.testing.assert_allclose(f[1], a[1], rtol=0, atol=1e-5)
