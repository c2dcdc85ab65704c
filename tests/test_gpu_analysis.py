"""Solvent analyses on the device against the reference's own functors
(Fourier_Autocorr.h, Vel_Autocorr_Fluid.h, recorded in
tests/golden/analysis_L6.npz) and against numpy restatements on the same
states."""
import os

import numpy as np
import pytest

from starpolymersmd_gb300 import analysis, capi, system
from tests import golden_replay as gr
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu


def _solvent_context(precision, L=6, n_c=5, shear=0.2):
    fpos, fvel = system.uniform_fluid((L, L, L), n_c, 1.0, np.random.default_rng(7))
    return H.context_for(None, fpos, fvel, L, 1.0, shear, 1, precision=precision,
                         rng=capi.RNG_PHILOX, seed=3)


def _numpy_modes(pos, vel, L):
    k = 2 * np.pi / L
    out = np.zeros((3, 3), dtype=np.complex128)
    for j in range(3):
        e = np.exp(1j * k * pos[:, j])
        out[j] = (vel * e[:, None]).sum(axis=0) / len(pos)
        out[j, j] = 0.0
    return out


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_fourier_modes_match_numpy(precision):
    L = 6
    with _solvent_context(precision, L) as ctx:
        fa = analysis.FourierAutocorr(3, 0.1)
        fb = analysis.FourierAutocorr(3, 0.1)
        for t in range(5):
            ctx.mpc_step(t, 0.1)
            p, v = ctx.get_fluid(0)
            got = ctx.fourier_modes(0, L)
            want = _numpy_modes(p, v, L)
            tol = 1e-12 if precision == capi.FP64 else 1e-6
            np.testing.assert_allclose(got, want, rtol=0, atol=tol * np.abs(v).max())
            assert np.all(np.diag(got) == 0)
            fa.push(got)
            fb.push(want)
        ta, aa = fa.result()
        tb, ab = fb.result()
        assert fa.counter == 3
        np.testing.assert_allclose(aa, ab, rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_velocity_autocorrelation_matches_numpy(precision):
    n_p, entries = 150, 4
    with _solvent_context(precision) as ctx:
        ctx.vacf_start(0, n_p, entries)
        window, sums, calcs = [], np.zeros(entries), 0
        for t in range(9):
            ctx.mpc_step(t, 0.1)
            ctx.vacf_sample()
            _, v = ctx.get_fluid(0)
            window.append(v[:n_p].copy())
            window = window[-entries:]
            if len(window) == entries:
                for j in range(entries):
                    sums[j] += np.sum(window[0] * window[j])
                calcs += 1
        got, n = ctx.vacf_result()
        assert n == calcs == 6
        np.testing.assert_allclose(got, sums, rtol=1e-12)
        avg = analysis.vacf_average(got, n, n_p)
        assert avg[0] > 0
        assert analysis.vacf_diffusion(avg, 1.0, n) == pytest.approx(
            np.sum(sums / n / n_p * 1.0 / n) / 3.0)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32], ids=["fp64", "fp32"])
def test_analyses_replay_reference(golden_dir, precision):
    # The reference's sheared solvent replayed on its own draws; after every
    # collision the device's Fourier modes and velocity samples are taken as
    # the reference's Fourier_Autocorr and Vel_Autocorr_Fluid took them over
    # every solvent particle. FP64: modes, autocorrelation and lag sums to
    # 1e-12; FP32: to FP32 accuracy.
    fx = gr.load(os.path.join(golden_dir, "analysis_L6.npz"))
    coll = gr.collision_index(fx)
    L = int(fx["L"][0])
    n_f = len(fx["fluid_pos0"])
    tol = 1e-12 if precision == capi.FP64 else 2e-5
    with H.fixture_context(fx, precision=precision) as ctx:
        fa = analysis.FourierAutocorr(int(fx["fourier_entries"]), float(fx["h"]))
        ctx.vacf_start(0, n_f, int(fx["vacf_entries"]))
        vscale = np.abs(fx["fluid_vel0"]).max()
        for t in range(int(fx["n_loop"])):
            k = coll[t]
            ctx.mpc_step(t, float(fx["h"]), fx["shift"][k], np.nan_to_num(fx["gamma"][k]),
                         fx["u_phi"][k], fx["u_theta"][k])
            modes = ctx.fourier_modes(0, L)
            np.testing.assert_allclose(modes, fx["fourier_modes"][k], rtol=0, atol=tol * vscale)
            fa.push(modes)
            ctx.vacf_sample()
        ctx.raise_on_device_error()
        assert fa.counter == int(fx["fourier_counter"])
        _, acf = fa.result()
        want = fx["fourier_acf"] / fa.counter
        np.testing.assert_allclose(acf.T, want, rtol=0, atol=tol * np.abs(want).max())
        sums, n = ctx.vacf_result()
        assert n == int(fx["vacf_counter"])
        np.testing.assert_allclose(sums, fx["vacf_lag_sums"], rtol=0,
                                   atol=tol * np.abs(fx["vacf_lag_sums"]).max())
