"""The MPC solvent against kinetic theory: the checks the reference's
results/plot_MPC_tests.py makes on its mpc-test runs (N_c = 10, h = 0.1,
rotation angle 130 degrees, kT = 1), here on the GPU paths.

  * Linear shear profile (plot_MPC_tests.py:59-60): a fluid started at rest
    under Lees-Edwards shear relaxes to v_x = shear * y.
  * Maxwell speed distribution at kT = 1 (plot_MPC_tests.py:82): a fluid
    started with the reference's uniform velocities (MPC.cpp:40-47, kT = 1/12)
    is brought to P(|v|) = 4 pi v^2 (2 pi)^(-3/2) exp(-v^2 / 2) by the cell
    thermostat and the collisions.
  * Transverse velocity autocorrelation (plot_MPC_tests.py:98-107): the
    transverse modes at k = 2 pi / L (Fourier_Autocorr) decay as
    exp(-nu k^2 t) with the kinematic viscosity nu = 0.8705 the reference
    plots against.
Fits carry standard errors from independent segments of the run; the
comparisons allow four of them plus a small model allowance, stated per test.
"""
import numpy as np
import pytest

from starpolymersmd_gb300 import capi

pytestmark = pytest.mark.gpu

NC, H_MPC = 10, 0.1
NU = 0.8705  # results/plot_MPC_tests.py:107


def _fluid(precision, L, shear, seed, reference_velocities):
    rep = dict(L=(L,) * 3, n_fluid=NC * L ** 3, kT=1.0, shear=shear, h=H_MPC, md_dt=H_MPC,
               seed=seed)
    # one collision per cycle; the reference's delrx advance is then the
    # physical one (MPC.cpp:117-119 with step_update = 1)
    ctx = capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX, step_update=1,
                       delrx_mode=capi.DELRX_REFERENCE, strict_cells=0)
    ctx.init_solvent(0, seed=seed, reference_velocities=reference_velocities)
    return ctx


def _segments_mean_se(values):
    v = np.asarray(values)
    return float(v.mean()), float(v.std(ddof=1) / np.sqrt(len(v)))


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32], ids=["fp64", "fp32"])
def test_linear_shear_profile(precision, record_property):
    L, shear = 20, 0.1
    with _fluid(precision, L, shear, 5, True) as ctx:
        # slowest shear mode relaxes in L^2 / (pi^2 nu) = 47 time units
        ctx.cycles(3000)
        slopes = []
        edges = np.arange(L + 1) - L / 2
        yc = 0.5 * (edges[1:] + edges[:-1])
        for seg in range(10):
            acc = np.zeros(L)
            cnt = np.zeros(L)
            for _ in range(30):
                ctx.cycles(10)
                p, v = ctx.get_fluid(0)
                k = np.clip(np.floor(p[:, 1] + L / 2).astype(int), 0, L - 1)
                acc += np.bincount(k, weights=v[:, 0], minlength=L)
                cnt += np.bincount(k, minlength=L)
            vx = acc / cnt
            slopes.append(((yc - yc.mean()) * (vx - vx.mean())).sum() / ((yc - yc.mean()) ** 2).sum())
        ctx.raise_on_device_error()
    m, se = _segments_mean_se(slopes)
    record_property("slope", (m, se))
    # statistical error plus 1 % for the model (stored positions are the
    # primary-box images right after a collision)
    assert abs(m - shear) < 4.0 * se + 0.01 * shear, (m, se)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32], ids=["fp64", "fp32"])
def test_maxwell_speed_distribution(precision, record_property):
    L = 30
    with _fluid(precision, L, 0.0, 9, True) as ctx:
        ctx.cycles(300)
        speeds = []
        for _ in range(3):
            ctx.cycles(50)
            _, v = ctx.get_fluid(0)
            speeds.append(np.linalg.norm(v, axis=1))
        ctx.raise_on_device_error()
    s = np.concatenate(speeds)
    edges = np.linspace(0.0, 5.0, 51)
    obs, _ = np.histogram(s, bins=edges)
    # expected counts: the Maxwell speed distribution integrated over each bin
    fine = np.linspace(0.0, 5.0, 5001)
    pdf = (2.0 * np.pi) ** -1.5 * 4.0 * np.pi * fine ** 2 * np.exp(-fine ** 2 / 2.0)
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(fine))])
    exp = len(s) * np.diff(np.interp(edges, fine, cdf))
    # three snapshots 50 collisions apart: treat as independent draws
    chi2 = float(((obs - exp) ** 2 / exp).sum())
    dof = len(obs) - 1
    record_property("chi2_dof", (chi2, dof))
    assert chi2 < dof + 6.0 * np.sqrt(2.0 * dof), chi2
    assert abs(float((s ** 2).mean()) / 3.0 - 1.0) < 0.01


@pytest.mark.parametrize("precision,n", [(capi.FP64, 40000), (capi.FP32, 80000)],
                         ids=["fp64", "fp32"])
def test_transverse_velocity_autocorrelation(precision, n, record_property):
    L = 30
    k2 = (2.0 * np.pi / L) ** 2
    with _fluid(precision, L, 0.0, 13, False) as ctx:
        ctx.cycles(200)
        modes = np.empty((n, 3, 3), dtype=np.complex128)
        for t in range(n):
            ctx.cycles(1)
            modes[t] = ctx.fourier_modes(0, L)
        ctx.raise_on_device_error()
    # lags up to where the theory has fallen to 0.3
    lag_max = int(np.log(1 / 0.3) / (NU * k2) / H_MPC)
    lags = np.arange(1, lag_max + 1)
    nus = []
    for seg in np.array_split(np.arange(n), 8):
        x = modes[seg]
        m = len(seg)
        c = np.zeros(lag_max + 1)
        for j in range(3):
            for d in range(3):
                if d == j:
                    continue  # transverse components only
                # no mean is subtracted: the mode's mean is zero at k != 0,
                # and subtracting a segment's own mean lowers the estimate by
                # about 2 tau / T (tau = 1 / (nu k^2)), which steepens the
                # normalised decay
                z = x[:, j, d]
                f = np.fft.fft(z, 2 * m)
                acf = np.fft.ifft(f * np.conj(f)).real[: lag_max + 1] / (m - np.arange(lag_max + 1))
                c += acf
        r = c[1:] / c[0]
        ok = r > 0.05
        t = lags[ok] * H_MPC
        a = -float((t * np.log(r[ok])).sum() / (t * t).sum())
        nus.append(a / k2)
    m, se = _segments_mean_se(nus)
    record_property("nu", (m, se))
    # four standard errors plus 3 % for the kinetic-theory formula itself
    assert abs(m - NU) < 4.0 * se + 0.03 * NU, (m, se, nus)
