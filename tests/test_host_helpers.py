"""Host-side helpers of the bench and the precision report (no GPU needed):
the algorithmic bytes the bench divides by, and the block-mean errors the
report quotes."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_bench_key_bytes_follow_the_packing_rule():
    # 32-bit keys for FP32 contexts whose boxes all have at most 65,536 cells
    import bench
    from starpolymersmd_gb300 import system
    small = [system.ReplicaSpec(L=40, arms=3, n_arm=10, solvophobic_fraction=0.5, shear=0.0,
                                seed=1)]
    big = small + [system.ReplicaSpec(L=41, arms=3, n_arm=10, solvophobic_fraction=0.5,
                                      shear=0.0, seed=2)]
    assert bench.key_bytes("fp32", small) == 4
    assert bench.key_bytes("fp32", big) == 8
    assert bench.key_bytes("fp64", small) == 8
    r = bench.kernel_rooflines({"fluid_bin": 1.0, "build_perm": 1.0, "collide": 1.0}, 1,
                               1000, 1100, 50, 32, 6000.0, kb=4)
    assert r["fluid_bin"]["algorithmic_bytes_per_launch"] == 1000 * 36
    assert r["build_perm"]["algorithmic_bytes_per_launch"] == 1100 * 8
    assert r["collide"]["algorithmic_bytes_per_launch"] == 1100 * 68 + 51 * 4


def test_precision_report_errors_from_block_means():
    import numpy as np
    from starpolymersmd_gb300 import precision_report as P
    x = np.repeat(np.arange(10.0), 5)  # ten blocks of five equal samples
    m, e = P._mean_err(x)
    assert m == 4.5
    assert np.isclose(e, np.arange(10.0).std(ddof=1) / np.sqrt(10))
