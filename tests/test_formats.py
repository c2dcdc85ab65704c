"""The reference's restart formats (starpolymersmd_gb300.formats) against the
reference's own writers and readers, run through the compiled reference
(oracle/refbuild): byte-identical files, identical doubles read back. Skipped
where the reference checkout is not available (its build needs the sources)."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from starpolymersmd_gb300 import formats, system


def _ref(L=6, n_c=3, shear=0.05, star=None):
    try:
        r = orc.RefSystem((L, L, L), 1.0, 1.0, n_c, shear, 1)
    except (FileNotFoundError, OSError) as e:
        pytest.skip(f"reference not available: {e}")
    if star:
        r.add_star(*star)
    r.mpc_initialize()
    return r


def test_fluid_text_is_the_reference_bytes(tmp_path):
    r = _ref()
    pos, vel = r.get_fluid()
    mine, theirs = str(tmp_path / "mine.dat"), str(tmp_path / "ref.dat")
    formats.write_fluid_complete(mine, pos, vel)
    r.print_fluid_complete(theirs)
    assert open(mine, "rb").read() == open(theirs, "rb").read()


@pytest.mark.parametrize("shear", [0.0, 0.05])
def test_fluid_reader_matches_the_reference(tmp_path, shear):
    # a file with one in-box line per particle: the reference's reader draws
    # no random numbers, so both readers must give the same doubles
    L, n_c = 6, 3
    r = _ref(L, n_c, shear)
    rng = np.random.default_rng(4)
    n = r.n_fluid
    pos = (rng.random((n, 3)) - 0.5) * (L - 1e-3)
    vel = rng.normal(size=(n, 3))
    path = str(tmp_path / "in.dat")
    with open(path, "w") as f:  # full precision, so the parse is the only rounding
        f.writelines(" ".join(repr(float(t)) for t in (*a, *b)) + "\n" for a, b in zip(pos, vel))
    r.initialize_fluid_from_file(path, (L, L, L))
    rp, rv = r.get_fluid()
    p, v, n_file, n_added = formats.read_fluid(path, n, (L, L, L), shear=shear)
    assert (n_file, n_added) == (n, 0)
    np.testing.assert_array_equal(p, rp)
    np.testing.assert_array_equal(v, rv)


def test_fluid_reader_refills_outside_and_missing_particles(tmp_path):
    L = (8, 8, 8)
    path = str(tmp_path / "in.dat")
    pos = np.array([[0.5, 1.0, -2.0], [10.0, 0.0, 0.0]])  # the second is outside
    formats.write_fluid_complete(path, pos, np.ones((2, 3)))
    p, v, n_file, n_added = formats.read_fluid(path, 5, L, L_old=(6, 8, 8),
                                               rng=np.random.default_rng(1))
    assert (n_file, n_added) == (1, 4)
    assert np.all(np.abs(p) <= 4.0)
    # the box grew along x by 2: refilled particles sit in the new slabs
    assert np.all(np.abs(p[1:, 0]) >= 3.0)
    np.testing.assert_allclose(v.mean(axis=0), 0.0, atol=1e-15)


def test_pdb_with_velocity_is_the_reference_bytes(tmp_path):
    A, B, arms, mass = 2, 3, 4, 5.0
    r = _ref(L=14, n_c=1, star=(A, B, arms, mass))
    m = r.get_monomers()
    amphi_t, anchor, src, dst = system.star_topology(arms, A, B)
    np.testing.assert_array_equal(m["amphi"], amphi_t)
    star = system.Star(arms, A, B, mass, m["pos"], m["vel"], amphi_t, anchor, src, dst)
    mine, theirs = str(tmp_path / "mine.pdb"), str(tmp_path / "ref.pdb")
    formats.write_pdb_with_velocity(mine, 7, [star])
    r.print_pdb_with_velocity(theirs, 7)
    assert open(mine, "rb").read() == open(theirs, "rb").read()


@pytest.mark.parametrize("set_zero", [False, True])
def test_star_pdb_reader_matches_the_reference(tmp_path, set_zero):
    A, B, arms, mass = 3, 2, 5, 5.0
    rng = np.random.default_rng(8)
    star = system.make_star(arms, A + B, B / (A + B), mass, 1.0, rng)
    star.pos += np.array([0.3, -0.7, 1.1])
    path = str(tmp_path / "star.pdb")
    formats.write_pdb_with_velocity(path, 0, [star])
    r = _ref(L=20, n_c=1, star=(A, B, arms, mass))
    r.star_from_file(0, path, A, B, arms, set_zero)
    m = r.get_monomers()
    rp, rv = m["pos"], m["vel"]
    got = formats.read_star_pdb(path, arms, A, B, mass=mass, set_zero=set_zero)
    np.testing.assert_array_equal(got.pos, rp)
    np.testing.assert_array_equal(got.vel, rv)
    # the format keeps three decimals
    if not set_zero:
        np.testing.assert_allclose(got.pos, star.pos, atol=5e-4 + 1e-12)


def test_pdb_models_of_many_stars_round_trip(tmp_path):
    sol = system.star_solution(3, 3, 4, 0.5, 5.0, 1.0, (12, 12, 12), np.random.default_rng(2))
    path = str(tmp_path / "traj.pdb")
    with open(path, "w") as f:
        formats.write_pdb_with_velocity(f, 0, sol.stars)
        formats.write_pdb_with_velocity(f, 10, sol.stars, pos=sol.pos + 0.25, vel=sol.vel)
    models = formats.read_pdb_models(path)
    assert [m[0] for m in models] == [0, 10]
    for (p, v), st in zip(models[1][1], sol.stars):
        np.testing.assert_allclose(p, st.pos + 0.25, atol=5e-4 + 1e-12)
        np.testing.assert_allclose(v, st.vel, atol=5e-4 + 1e-12)
