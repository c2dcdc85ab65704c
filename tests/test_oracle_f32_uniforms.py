"""The oracle's FP32-uniform mode draws what the FP32 kernels draw.

In this mode the collision's rotation axes and gamma variates come from the
23-bit uniforms (w >> 9) 2^-23 + 2^-24 of the same Philox words the FP32
kernels use (the grid shift keeps the 53-bit uniforms, as the kernels do).
Pinned here by a Python restatement of the draws (Philox words from the
oracle's known-answer-tested generator, Marsaglia-Tsang in numpy) injected
into a second oracle: both runs must agree bit for bit.
"""
import numpy as np

from oracle import oracle as orc
from starpolymersmd_gb300 import system


def _u23(w):
    return float(int(w) >> 9) * 2.0 ** -23 + 2.0 ** -24


def _u53(lo, hi):
    return float(((int(hi) << 32) | int(lo)) >> 11) * 2.0 ** -53 + 2.0 ** -54


def _words(seed, cell, step, k):
    return orc.philox4x32_10((cell, step & 0xFFFFFFFF, step >> 32, k),
                             (seed & 0xFFFFFFFF, seed >> 32))


def _gamma23(seed, step, cell, shape):
    # Marsaglia & Tsang (2000) on the 23-bit uniforms: normal from block
    # 1 + 2i by Box-Muller, acceptance uniform from block 2 + 2i
    d = shape - 1.0 / 3.0
    c = 1.0 / np.sqrt(9.0 * d)
    for it in range(64):
        w = _words(seed, cell, step, 1 + 2 * it)
        a, b = _u23(w[1]), _u23(w[3])
        x = np.sqrt(-2.0 * np.log(a)) * np.cos(2.0 * np.pi * b)
        v = 1.0 + c * x
        if v <= 0.0:
            continue
        v = v * v * v
        u = _u23(_words(seed, cell, step, 2 + 2 * it)[1])
        x2 = x * x
        if u < 1.0 - 0.0331 * (x2 * x2) or np.log(u) < 0.5 * x2 + d * (1.0 - v + np.log(v)):
            return d * v
    return d


def test_f32_uniform_mode_equals_injected_restatement():
    L, seed, step, kT = 5, 97, 3, 1.3
    rng = np.random.default_rng(12)
    fpos, fvel = system.uniform_fluid((L, L, L), 10, kT, rng)
    a = orc.OracleSystem((L, L, L), kT, 0.1, 1, len(fpos))
    a.set_fluid(fpos, fvel)
    a.set_philox(seed, step)
    a.set_f32_uniforms(True)
    a.mpc_step(0, 0.1)
    assert a.error() == 0
    tot, _ = a.cell_counts()
    # the same collision with the draws restated above injected
    w0, w1 = _words(seed, 0xFFFFFFFF, step, 0), _words(seed, 0xFFFFFFFF, step, 1)
    shift = np.array([_u53(w0[0], w0[1]), _u53(w0[2], w0[3]), _u53(w1[0], w1[1])]) - 0.5
    n = len(tot)
    uphi, uth, gam = np.zeros(n), np.zeros(n), np.zeros(n)
    for c in range(n):
        w = _words(seed, c, step, 0)
        uphi[c], uth[c] = _u23(w[1]), _u23(w[3])
        if tot[c] >= 2:
            gam[c] = _gamma23(seed, step, c, 1.5 * (int(tot[c]) - 1)) * kT
    b = orc.OracleSystem((L, L, L), kT, 0.1, 1, len(fpos))
    b.set_fluid(fpos, fvel)
    b.set_inject(shift, gam, uphi, uth)
    b.mpc_step(0, 0.1)
    assert b.error() == 0
    pa, va = a.get_fluid()
    pb, vb = b.get_fluid()
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(va, vb)
    fa, _ = a.cell_members()
    fb, _ = b.cell_members()
    np.testing.assert_array_equal(fa, fb)


def test_f32_uniform_mode_changes_only_the_draws():
    # same shift (53-bit); the 23-bit uniforms are the top bits of the same
    # words, so axes and gamma variates move by ~2^-23 relative: same cells,
    # velocities apart by ~1e-6, momentum of every cell conserved in both modes
    L = 6
    rng = np.random.default_rng(3)
    fpos, fvel = system.uniform_fluid((L, L, L), 10, 1.0, rng)
    out = []
    for f32 in (False, True):
        o = orc.OracleSystem((L, L, L), 1.0, 0.0, 1, len(fpos))
        o.set_fluid(fpos, fvel)
        o.set_philox(5, 0)
        o.set_f32_uniforms(f32)
        o.mpc_step(0, 0.1)
        p, v = o.get_fluid()
        fc, _ = o.cell_members()
        out.append((p, v, fc))
        mom = np.zeros((L ** 3, 3))
        np.add.at(mom, fc, v)
        mom0 = np.zeros((L ** 3, 3))
        np.add.at(mom0, fc, fvel)
        np.testing.assert_allclose(mom, mom0, atol=1e-12)
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][2], out[1][2])
    dv = np.abs(out[0][1] - out[1][1]).max()
    assert 0.0 < dv < 1e-4
