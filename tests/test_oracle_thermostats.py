"""The oracle's MPC-off thermostats on the CPU: the Lowe-Andersen restatement
(Lowe_Andersen.cpp:28-88) exchanges momentum pairwise, so the star's total
momentum is conserved, and it brings a cold star to the target temperature;
the Andersen restatement (Andersen_stochastic.cpp:30-59) holds the
temperature too."""
import numpy as np

from oracle import oracle as orc
from starpolymersmd_gb300 import system


def _star(seed, arms=8, n_arm=12, L=24):
    rng = np.random.default_rng(seed)
    for _ in range(200):
        st = system.make_star(arms, n_arm, 0.5, 5.0, 1.0, rng, bond=1.01, outward_bias=0.0)
        if np.abs(st.pos).max() < L / 2 - 1.5:
            return st, L
    raise RuntimeError("no compact star")


def _oracle(st, L):
    n = st.n
    o = orc.OracleSystem((L, L, L), 1.0, 0.0, 1000, 0, n, mol_start=[0, n])
    o.set_monomers(st.pos, st.vel * 0.1, np.zeros_like(st.pos), np.full(n, st.mass), st.amphi,
                   st.anchor)
    o.set_bonds(st.bond_src, st.bond_dst)
    return o


def _temperature(v, m):
    u = v - v.mean(axis=0)
    return m * (u * u).sum() / (3 * (len(v) - 1))


def test_lowe_andersen_conserves_momentum_and_thermalises():
    st, L = _star(4)
    o = _oracle(st, L)
    o.set_lowe_andersen(20.0, 1.5, 11)
    o.init_md()
    p0 = st.mass * o.get_monomers()[1].sum(axis=0)
    temps = []
    for t in range(3000):
        o.propagate(False)
        if t % 50 == 49:
            temps.append(_temperature(o.get_monomers()[1], st.mass))
    assert o.error() == 0
    p1 = st.mass * o.get_monomers()[1].sum(axis=0)
    assert np.abs(p1 - p0).max() < 1e-10
    assert abs(np.mean(temps[20:]) - 1.0) < 0.12


def test_andersen_holds_the_temperature():
    st, L = _star(5)
    o = _oracle(st, L)
    o.set_andersen(5.0, 13)
    o.init_md()
    temps = []
    for t in range(3000):
        o.propagate(False)
        if t % 50 == 49:
            temps.append(_temperature(o.get_monomers()[1], st.mass))
    assert o.error() == 0
    assert abs(np.mean(temps[20:]) - 1.0) < 0.12
