"""The C restatement oracle reproduces the reference bit for bit.

The fixtures in tests/golden were produced by the reference's own sources
(tests/golden/make_golden.py); replaying the same initial state and the same
recorded draws through oracle/smpc_oracle.c must give identical doubles for
every particle, cell occupancy, Lees-Edwards offset, potential energy and
temperature.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests import golden_replay as gr

FIXTURES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def make_oracle(fx):
    n_f = len(fx["fluid_pos0"])
    n_m = len(fx["mono_pos0"]) if gr.has_star(fx) else 0
    o = orc.OracleSystem(fx["L"], float(fx["kT"]), float(fx["shear"]), int(fx["step_update"]),
                         n_f, n_m, mol_start=[0, n_m] if n_m else [0], lambda_=float(fx["lam"]),
                         md_dt=float(fx["md_dt"]), angular_momentum=int(fx.get("amc", 0)))
    o.set_fluid(fx["fluid_pos0"], fx["fluid_vel0"])
    if n_m:
        o.set_monomers(fx["mono_pos0"], fx["mono_vel0"], fx["mono_force0"], fx["mono_mass"],
                       fx["mono_amphi"], fx["mono_anchor"])
        o.set_bonds(fx["bond_src"], fx["bond_dst"])
        if gr.is_andersen(fx):
            o.set_andersen(float(fx["andersen_nu"]), 0)
        o.init_md()
    return o


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_matches_reference_bitwise(path):
    fx = gr.load(path)
    o = make_oracle(fx)
    if gr.has_star(fx):
        _, _, f0 = o.get_monomers()
        np.testing.assert_array_equal(f0, fx["mono_force0"])
    coll = gr.collision_index(fx)
    for t in range(int(fx["n_loop"])):
        if gr.has_star(fx) and int(fx["with_md"]):
            if gr.is_andersen(fx):
                o.stage_andersen(*gr.andersen_resets(fx, t))
            o.propagate(True)
            assert o.epot() == fx["epot"][t]
        if not int(fx["md_only"]):
            k = coll.get(t)
            if k is not None:
                o.set_inject(fx["shift"][k], fx["gamma"][k], fx["u_phi"][k], fx["u_theta"][k])
            o.mpc_step(t, float(fx["h"]))
            assert o.error() == 0
            if k is not None:
                tot, fl = o.cell_counts()
                np.testing.assert_array_equal(tot, fx["count_total"][k])
                np.testing.assert_array_equal(fl, fx["count_fluid"][k])
                p, v = o.get_fluid()
                np.testing.assert_array_equal(p, fx["fluid_pos"][k])
                np.testing.assert_array_equal(v, fx["fluid_vel"][k])
                assert o.temperature() == fx["temperature"][k]
        assert o.delrx == fx["delrx"][t]
        if gr.has_star(fx):
            p, v, f = o.get_monomers()
            np.testing.assert_array_equal(p, fx["mono_pos"][t])
            np.testing.assert_array_equal(v, fx["mono_vel"][t])
            np.testing.assert_array_equal(f, fx["mono_force"][t])


def test_topology_matches_reference_builder(golden_dir):
    from starpolymersmd_gb300 import system
    fx = gr.load(os.path.join(golden_dir, "star_mpc_L12.npz"))
    amphi, anchor, src, dst = system.star_topology(3, 2, 2)
    np.testing.assert_array_equal(amphi, fx["mono_amphi"])
    np.testing.assert_array_equal(anchor, fx["mono_anchor"])
    np.testing.assert_array_equal(src, fx["bond_src"])
    np.testing.assert_array_equal(dst, fx["bond_dst"])


# Published known-answer vectors for Philox4x32-10 (Random123 kat_vectors).
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_oracle_philox_known_answers(ctr, key, expect):
    np.testing.assert_array_equal(orc.philox4x32_10(ctr, key), np.array(expect, dtype=np.uint32))


def test_oracle_gamma_moments():
    # Gamma(a, 1) has mean a and variance a; 10^4 samples per shape.
    for a in (1.5, 13.5, 45.0):
        g = np.array([orc.philox_gamma(11, s, c, a) for s in range(20) for c in range(500)])
        assert abs(g.mean() - a) < 4 * np.sqrt(a / g.size)
        assert abs(g.var() / a - 1.0) < 0.05


def test_recentre_fixture_exercises_check_bounds(golden_dir):
    # The star starts 3.5 cells off-centre; MPC::check_bounds must pull star 0's
    # centre of mass back to the origin at the first collision.
    fx = gr.load(os.path.join(golden_dir, "recentre_L12.npz"))
    assert np.abs(fx["mono_pos0"].mean(axis=0)).max() > 1.0
    assert np.abs(fx["mono_pos"][0].mean(axis=0)).max() < 0.1


def test_fourier_bookkeeping_matches_reference(golden_dir):
    # The host side of the Fourier autocorrelation (the window of samples and
    # the sums, starpolymersmd_gb300/analysis.py) fed the reference's own
    # modes gives the reference's Autocorrelation and calculation count
    # (Fourier_Autocorr.h:58-100).
    from starpolymersmd_gb300 import analysis
    fx = gr.load(os.path.join(golden_dir, "analysis_L6.npz"))
    fa = analysis.FourierAutocorr(int(fx["fourier_entries"]), float(fx["h"]))
    for m in fx["fourier_modes"]:
        fa.push(m)
    assert fa.counter == int(fx["fourier_counter"])
    _, acf = fa.result()
    np.testing.assert_allclose(acf.T * fa.counter, fx["fourier_acf"], rtol=1e-13, atol=1e-18)
