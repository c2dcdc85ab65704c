"""The identities behind the FP64 kernels' integer tests and FP32 pre-tests
(no GPU needed).

On GB300 every FP64 compare issues on the narrow FP64 pipe, so the FP64
kernels decide some comparisons on the bit patterns instead, and the
cluster MD decides most pair distances in FP32 before any FP64 work:

* ``not_negative(x)`` (csrc/mpc_kernels.cuh): x >= 0 for every double is
  "bits <= 0x7FF0000000000000 (+0 .. +inf) or bits == 0x8000000000000000
  (-0)";
* ``finite_bits(x)``: isfinite(x) is "exponent field != 0x7FF";
* ``r2_below(r2, c)`` (csrc/md_kernels.cuh): for a squared distance r2 (+0
  or more, or NaN) and a cut-off c > 0, r2 < c is the unsigned order of the
  bit patterns;
* the FP32 range test of the compacted pair forces and the FP32 membership
  test of the rebuild: with coordinates below 4096 in magnitude, r^2 computed
  from FP32-rounded coordinates lies within 2^-7 of the cut-off's value of
  the FP64 r^2, so a pair the FP32 test drops has a zero FP64 force, and a
  membership decided in FP32 outside the band is the FP64 one.
"""
import numpy as np

U64 = np.uint64


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.uint64)


def not_negative(x):
    b = bits(x)
    return (b <= U64(0x7FF0000000000000)) | (b == U64(0x8000000000000000))


def finite_bits(x):
    return ((bits(x) >> U64(52)) & U64(0x7FF)) != U64(0x7FF)


def r2_below(r2, c):
    return bits(r2) < bits(c)


def edge_doubles():
    specials = [0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324,
                2.2250738585072014e-308, -2.2250738585072014e-308, 1.7976931348623157e308,
                -1.7976931348623157e308]
    neg_nan = np.array([0xFFF8000000000000, 0xFFF0000000000001, 0x7FF0000000000001],
                       dtype=np.uint64).view(np.float64)
    rng = np.random.default_rng(7)
    random_bits = rng.integers(0, 2**64, size=200_000, dtype=np.uint64).view(np.float64)
    return np.concatenate([np.array(specials), neg_nan, random_bits])


def test_sign_and_finiteness_on_the_bits():
    x = edge_doubles()
    with np.errstate(invalid="ignore"):
        assert np.array_equal(not_negative(x), x >= 0.0)
    assert np.array_equal(finite_bits(x), np.isfinite(x))


def test_cutoff_compare_on_the_bits():
    rng = np.random.default_rng(11)
    # squared distances: +0, subnormals, normals around the cut-offs, +inf, NaNs
    r2 = np.concatenate([
        np.array([0.0, 5e-324, 1e-300, np.inf, np.nan]),
        np.array([0x7FF8000000000000, 0xFFF8000000000000], dtype=np.uint64).view(np.float64),
        rng.uniform(0.0, 10.0, 100_000),
        rng.exponential(1.0, 100_000),
    ])
    for c in (1.0594631, 2.25, 1.2599210498948732, 6.25, 20.25):
        cut = np.full_like(r2, c)
        near = np.concatenate([np.nextafter(cut[:50], 0.0), cut[:50], np.nextafter(cut[:50], 10.0)])
        for v in (r2, near):
            with np.errstate(invalid="ignore"):
                assert np.array_equal(r2_below(v, np.full_like(v, c)), v < c)


def fp32_r2(xi, xj):
    # the kernels' FP32 form: coordinates rounded to FP32, differences and
    # fmaf(d0, d0, fmaf(d1, d1, d2 * d2)) in FP32
    f = np.float32
    d = xj.astype(f) - xi.astype(f)
    d0, d1, d2 = d[:, 0].astype(np.float64), d[:, 1].astype(np.float64), d[:, 2].astype(np.float64)
    t = (d2 * d2).astype(f).astype(np.float64)
    t = (d1 * d1 + t).astype(f).astype(np.float64)
    return (d0 * d0 + t).astype(f).astype(np.float64)


def test_fp32_range_tests_keep_a_margin():
    rng = np.random.default_rng(3)
    n = 400_000
    for scale in (25.0, 600.0, 4095.0):
        xi = rng.uniform(-scale, scale, (n, 3))
        xj = xi + rng.uniform(-2.9, 2.9, (n, 3))
        d = xj - xi
        r2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]  # FP64, the reference's form
        r2f = fp32_r2(xi, xj)
        # force cut-offs (widened by 2^-7) and the Verlet radius (band of 2^-7)
        for c in (1.0594631, 1.2599210498948732, 2.25, 6.25, 2.8 ** 2):
            near = np.abs(r2 - c) < 0.5
            err = np.abs(r2f[near] - r2[near]).max()
            assert err < c * 2.0 ** -7 / 4, (scale, c, err)
            # no pair inside the cut-off is dropped by the widened FP32 test
            inside = r2 < c
            assert np.all(r2f[inside] < np.float32(c) * np.float32(1.0 + 2.0 ** -7))
