"""smpc_temperature_all_noalloc, called through the C ABI, against
smpc_temperature_all on the same context: two calls in a row, and again after
the state has moved on. Named to run last, after every other GPU test has
used the device; it passes on its own as well."""
import ctypes as C

import numpy as np
import pytest

from starpolymersmd_gb300 import capi, system

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # both paths sum the same FP64 partials in the same order


def _noalloc(ctx):
    out = np.full(ctx.n_rep, np.nan)
    rc = ctx.lib.smpc_temperature_all_noalloc(ctx.h, out.ctypes.data_as(C.c_void_p))
    assert rc == 0, ctx.lib.smpc_last_error(ctx.h)
    return out


def _solvent_boxes(precision):
    rng = np.random.default_rng(17)
    reps, states = [], []
    for k, L in enumerate((6, 9, 12)):
        fp, fv = system.uniform_fluid((L, L, L), 10, 1.0, rng)
        reps.append(dict(L=(L, L, L), n_fluid=len(fp), kT=1.0, shear=0.01 * (k + 1), h=0.1,
                         seed=70 + k))
        states.append((fp, fv))
    ctx = capi.Context(reps, precision=precision, rng=capi.RNG_PHILOX, step_update=1)
    for k, (fp, fv) in enumerate(states):
        ctx.set_fluid(k, fp, fv)
    return ctx


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32], ids=["fp64", "fp32"])
def test_noalloc_temperature_matches_temperature_all(precision):
    with _solvent_boxes(precision) as ctx:
        ctx.cycles(2)
        for _ in range(2):
            ref = ctx.temperature_all()
            a = _noalloc(ctx)
            b = _noalloc(ctx)
            np.testing.assert_allclose(a, ref, rtol=RTOL)
            np.testing.assert_allclose(b, ref, rtol=RTOL)
            assert np.all(np.abs(ref - 1.0) < 0.5)
            ctx.cycles(3)
        ctx.raise_on_device_error()


def test_noalloc_temperature_rejects_contexts_beyond_its_scratch():
    reps = [dict(L=(2, 2, 2), n_fluid=8, kT=1.0, h=0.1, seed=k) for k in range(4097)]
    with capi.Context(reps, precision=capi.FP32, rng=capi.RNG_PHILOX) as ctx:
        out = np.zeros(ctx.n_rep)
        rc = ctx.lib.smpc_temperature_all_noalloc(ctx.h, out.ctypes.data_as(C.c_void_p))
        assert rc == 5  # SMPC_E_UNSUPPORTED
        assert b"4096 replicas" in ctx.lib.smpc_last_error(ctx.h)
