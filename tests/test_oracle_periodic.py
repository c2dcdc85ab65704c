"""The oracle's periodic many-molecule MD (CPU only).

Pinned in the one-star limit to the reference's own fixtures: a star away
from the faces sees no periodic image, so the periodic form must replay the
reference's MD up to the order of the force sums. Checked beyond that limit
by conservation laws: total force zero (pairs and bonds under the
Lees-Edwards minimum image are antisymmetric) and energy conservation of the
velocity-Verlet integrator at a small time step with stars across the faces.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from starpolymersmd_gb300 import system
from tests import golden_replay as gr

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _close(a, b, rtol):
    scale = max(1.0, float(np.abs(b).max()))
    np.testing.assert_allclose(a, b, rtol=rtol, atol=rtol * scale)


@pytest.mark.parametrize("name", ["star_mpc_L12", "md_saw_L16"])
def test_periodic_oracle_replays_one_star_fixture(name):
    fx = gr.load(os.path.join(GOLDEN, name + ".npz"))
    n_m = len(fx["mono_pos0"])
    su = int(fx["step_update"])
    o = orc.OracleSystem(fx["L"], float(fx["kT"]), float(fx["shear"]), su,
                         len(fx["fluid_pos0"]), n_m, mol_start=[0, n_m],
                         lambda_=float(fx["lam"]), md_dt=float(fx["md_dt"]), mono_wrap=1)
    o.set_fluid(fx["fluid_pos0"], fx["fluid_vel0"])
    o.set_monomers(fx["mono_pos0"], fx["mono_vel0"], fx["mono_force0"], fx["mono_mass"],
                   fx["mono_amphi"], fx["mono_anchor"])
    o.set_bonds(fx["bond_src"], fx["bond_dst"])
    o.set_periodic_md(float(fx["h"]))
    o.init_md()
    _, _, f0 = o.get_monomers()
    _close(f0, fx["mono_force0"], 1e-12)
    coll = gr.collision_index(fx)
    for t in range(int(fx["n_loop"])):
        o.propagate(True)
        _close(o.epot(), fx["epot"][t], 1e-12)
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
        assert o.delrx == fx["delrx"][t]
        p, v, f = o.get_monomers()
        _close(p, fx["mono_pos"][t], 1e-12)
        _close(v, fx["mono_vel"][t], 1e-12)
        _close(f, fx["mono_force"][t], 1e-11)


def _solution_oracle(shear, md_dt, L=12, seed=1):
    sol = system.star_solution(4, 3, 5, 0.5, 5.0, 1.0, (L, L, L), np.random.default_rng(seed))
    o = orc.OracleSystem((L, L, L), 1.0, shear, 1000, 0, sol.n, mol_start=sol.mol_start,
                         md_dt=md_dt, delrx_dt_scale=1.0 / 1000, mono_wrap=1)
    o.set_monomers(sol.pos, sol.vel, np.zeros_like(sol.pos), sol.mass, sol.amphi, sol.anchor)
    o.set_bonds(sol.bond_src, sol.bond_dst)
    o.set_periodic_md(0.1)
    o.init_md()
    return sol, o


@pytest.mark.parametrize("shear", [0.0, 2.0])
def test_periodic_forces_sum_to_zero(shear):
    sol, o = _solution_oracle(shear, 0.002)
    for t in range(1, 101):
        o.propagate(False)
        o.mpc_step(t, 0.1)  # delrx advance only
    p, _, f = o.get_monomers()
    assert np.abs(p).max() <= 6.0
    assert np.abs(f.sum(axis=0)).max() < 1e-9 * np.abs(f).max() * len(f)
    assert o.delrx != 0.0 or shear == 0.0


def test_periodic_md_conserves_energy_at_small_step():
    # no shear: the periodic box is closed, stars across its faces
    sol, o = _solution_oracle(0.0, 0.002)
    p0, _, _ = o.get_monomers()
    energies = []
    for t in range(1, 601):
        o.propagate(True)
        if t % 100 == 0:
            _, v, _ = o.get_monomers()
            energies.append(0.5 * (sol.mass[:, None] * v * v).sum() + o.epot())
    e = np.array(energies)
    assert np.abs(e - e[0]).max() < 1e-3 * abs(e[0])
    p, _, _ = o.get_monomers()
    assert np.abs(p).max() <= 6.0


def test_star_solution_is_self_avoiding_across_images():
    L = 14
    sol = system.star_solution(5, 4, 6, 0.5, 5.0, 1.0, (L, L, L), np.random.default_rng(9))
    assert sol.n == 5 * (1 + 4 * 6)
    np.testing.assert_array_equal(sol.mol_start, np.arange(6) * 25)
    p = sol.pos
    d = p[:, None, :] - p[None, :, :]
    d -= L * np.round(d / L)
    r2 = (d * d).sum(axis=2)
    bonded = np.zeros_like(r2, dtype=bool)
    bonded[sol.bond_src, sol.bond_dst] = True
    bonded |= bonded.T
    np.fill_diagonal(bonded, True)
    assert r2[~bonded].min() > 1.0
    # bonds stay within each star
    ms = sol.mol_start
    mol = np.searchsorted(ms, np.arange(sol.n), side="right") - 1
    np.testing.assert_array_equal(mol[sol.bond_src], mol[sol.bond_dst])


@pytest.mark.parametrize("shear", [0.0, 1.5])
def test_periodic_grid_partners_match_all_pairs(shear):
    # the cell-grid partner search of large boxes gives the loop over all
    # monomers to the last bit, Lees-Edwards rows included
    sol, o = _solution_oracle(shear, 0.002, L=12, seed=6)
    for t in range(1, 301):
        o.propagate(False)
        o.mpc_step(t, 0.1)
    assert o.delrx != 0.0 or shear == 0.0
    np.testing.assert_array_equal(o.periodic_forces(True), o.periodic_forces(False))
