"""The device error word, raised by states set up on the host.

Each case maps to one of the reference's fatal paths or to a capacity of
this implementation, and is prepared from the host with ordinary inputs (no
kernel is made to fault): the kernels record the first offender and carry on
within their bounds, and smpc_error_word reports and clears the word.
  * a monomer outside the box with the reference's unwrapped monomer binning
    (MPC.cpp:227-234 prints and raises SIGSEGV): SMPC_ERR_MONO_CELL with the
    replica and the monomer;
  * a FENE bond stretched past R0 (Potentials.h:29,50, where the reference's
    force changes sign): SMPC_ERR_FENE with the two beads;
  * a Verlet list capacity too small for a compact star: SMPC_ERR_NEIGHBOR_OVF
    with the bead and the number of neighbours it has;
  * a solvent velocity beyond the FP32 path's fixed-point range:
    SMPC_ERR_FIXPOINT with the cell.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from starpolymersmd_gb300 import capi, system
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

ERR_MONO_CELL, ERR_NEIGHBOR_OVF, ERR_FENE, ERR_FIXPOINT = 2, 4, 64, 256


def _draws(L, rng):
    n = L ** 3
    return np.zeros(3), rng.gamma(13.5, 1.0, n), rng.random(n), rng.random(n)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_monomer_outside_the_box_reference_binning(precision):
    # molecule 0 (two bonded beads at the origin) decides the recentring; a
    # third, unbonded bead sits 3 cells beyond the +z face, so it stays out
    # of the box after MPC::check_bounds and its cell index is past the last
    L = 8
    rng = np.random.default_rng(5)
    fpos, fvel = system.uniform_fluid((L,) * 3, 10, 1.0, rng, reference_velocities=True)
    mpos = np.array([[0.0, 0.0, 0.0], [0.97, 0.0, 0.0], [0.0, 0.0, L / 2 + 3.0]])
    mvel = np.zeros((3, 3))
    rep = dict(L=(L,) * 3, n_fluid=len(fpos), n_mono=3, mol0_size=2, kT=1.0, shear=0.0,
               h=0.1, md_dt=0.01)
    with capi.Context([rep], precision=precision, rng=capi.RNG_INJECT, step_update=1,
                      mono_bin=capi.MONOBIN_REFERENCE, strict_cells=1) as ctx:
        ctx.set_fluid(0, fpos, fvel)
        ctx.set_monomers(0, mpos, mvel, np.zeros((3, 3)), np.full(3, 5.0), np.zeros(3, np.int32),
                         np.zeros(3, np.int32))
        ctx.set_bonds(0, [0], [1])
        ctx.init_md()
        word, info = ctx.error_word()
        assert word == 0
        ctx.mpc_step(0, 0.1, *_draws(L, rng))
        word, info = ctx.error_word()
        assert word & ERR_MONO_CELL, hex(word)
        assert list(info) == [ERR_MONO_CELL, 0, 2]
        word, _ = ctx.error_word()
        assert word == 0  # read and cleared
    # the oracle (the reference's sort) flags the same monomer cell error
    o = orc.OracleSystem((L,) * 3, 1.0, 0.0, 1, len(fpos), 3, mol_start=[0, 2, 3])
    o.set_fluid(fpos, fvel)
    o.set_monomers(mpos, mvel, np.zeros((3, 3)), np.full(3, 5.0), np.zeros(3, np.int32),
                   np.zeros(3, np.int32))
    o.set_bonds([0], [1])
    o.set_inject(*_draws(L, rng))
    o.mpc_step(0, 0.1)
    assert o.error() & 2  # ORC_ERR_MONO_CELL


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_fene_bond_beyond_r0(precision):
    # a plain (not anchor) bond; the reference preset's FENE (Potentials.h:24-55)
    L = 8
    rng = np.random.default_rng(8)
    fpos, fvel = system.uniform_fluid((L,) * 3, 10, 1.0, rng)
    rep = dict(L=(L,) * 3, n_fluid=len(fpos), n_mono=2, mol0_size=2, kT=1.0, shear=0.0, h=0.1,
               md_dt=0.01)

    def run(sep):
        mpos = np.array([[0.0, 0.0, 0.0], [sep, 0.0, 0.0]])
        with capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX,
                          step_update=10) as ctx:
            ctx.set_fluid(0, fpos, fvel)
            ctx.set_monomers(0, mpos, np.zeros((2, 3)), np.zeros((2, 3)), np.full(2, 5.0),
                             np.zeros(2, np.int32), np.zeros(2, np.int32))
            ctx.set_bonds(0, [0], [1])
            ctx.init_md()
            ctx.md_substeps(1)
            return ctx.error_word()

    word, info = run(1.6)  # R0 = 1.5 (Potentials.h:29)
    assert word & ERR_FENE, hex(word)
    assert info[0] == ERR_FENE and sorted(info[1:]) == [0, 1]
    word, _ = run(1.2)
    assert word == 0


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32])
def test_verlet_list_capacity(precision, periodic):
    L = 12
    star, fpos, fvel = H.small_star_system(L=L, arms=4, n_arm=8, shear=0.0, seed=6)
    rep = dict(L=(L,) * 3, n_fluid=len(fpos), n_mono=star.n, mol0_size=star.n, kT=1.0,
               shear=0.0, h=0.1, md_dt=0.01,
               flags=capi.REPLICA_PERIODIC_MD if periodic else 0)
    # neighbours within r_verlet = 2 of every bead, counted on the host
    d = np.linalg.norm(star.pos[:, None, :] - star.pos[None, :, :], axis=2)
    counts = (d <= 2.0).sum(axis=1) - 1
    cap = 3
    assert counts.max() > cap
    with capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX, step_update=10,
                      max_neighbors=cap,
                      mono_bin=capi.MONOBIN_WRAPPED if periodic else capi.MONOBIN_REFERENCE) as ctx:
        ctx.set_fluid(0, fpos, fvel)
        ctx.set_monomers(0, star.pos, star.vel, np.zeros_like(star.pos),
                         np.full(star.n, star.mass), star.amphi, star.anchor)
        ctx.set_bonds(0, star.bond_src, star.bond_dst)
        ctx.init_md()
        ctx.md_substeps(1)
        word, info = ctx.error_word()
        assert word & ERR_NEIGHBOR_OVF, hex(word)
        assert info[0] == ERR_NEIGHBOR_OVF
        bead = int(info[1])
        assert 0 <= bead < star.n and counts[bead] > cap
    with capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX, step_update=10,
                      max_neighbors=int(counts.max()) + 16,
                      mono_bin=capi.MONOBIN_WRAPPED if periodic else capi.MONOBIN_REFERENCE) as ctx:
        ctx.set_fluid(0, fpos, fvel)
        ctx.set_monomers(0, star.pos, star.vel, np.zeros_like(star.pos),
                         np.full(star.n, star.mass), star.amphi, star.anchor)
        ctx.set_bonds(0, star.bond_src, star.bond_dst)
        ctx.init_md()
        ctx.md_substeps(1)
        assert ctx.error_word()[0] == 0


@pytest.mark.parametrize("amc", [False, True])
def test_fixed_point_range_fp32(amc):
    # The FP32 cell sums are exact int64 fixed point for terms below 4095: the
    # fast-path kernel sums m v and m |v|^2 / 256 (|v| < 1024 at m = 1), the
    # generic kernel (angular-momentum-conserving collisions) m v and
    # m |v - c|^2 (|v - c| < 64 at m = 1). A particle beyond that is
    # reported, not clamped silently.
    L = 6
    rng = np.random.default_rng(2)
    fpos, fvel = system.uniform_fluid((L,) * 3, 10, 1.0, rng)
    rep = dict(L=(L,) * 3, n_fluid=len(fpos), kT=1.0, shear=0.0, h=0.1, seed=3)
    inside = 30.0 if amc else 900.0
    for v0, expect in ((inside, 0), (2000.0, ERR_FIXPOINT)):
        vel = fvel.copy()
        vel[7] = (v0, 0.0, 0.0)
        with capi.Context([rep], precision=capi.FP32, rng=capi.RNG_PHILOX, step_update=1,
                          strict_cells=0, angular_momentum=amc) as ctx:
            ctx.set_fluid(0, fpos, vel)
            ctx.mpc_step(0, 0.1)
            word, info = ctx.error_word()
            assert (word & ERR_FIXPOINT) == expect, (v0, hex(word))
            if expect:
                assert info[0] == ERR_FIXPOINT and 0 <= info[1] < L ** 3
