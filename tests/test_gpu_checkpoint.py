"""Checkpoint / restart through the C ABI (smpc_checkpoint_*).

A context restored from a checkpoint into a freshly created context with the
same replicas and options continues the run as if it had never stopped: on
the FP32 path, whose per-cell sums are exact fixed point, to the last bit;
on the FP64 path, whose per-cell sums run in the order the binning atomics
ranked the particles (so two runs of the same context already differ in the
last bits), within the FP64 tolerance. The solvent, the monomers, delrx, the
Philox collision counter and the Verlet bookkeeping all come back. Both the
batched single-star layout and a periodic many-star box are covered, through
memory and through a file; a checkpoint of other replicas is refused and
leaves the context as it was.
"""
import os

import numpy as np
import pytest

from starpolymersmd_gb300 import capi, system
from tests import gpu_helpers as H
from tests.test_gpu_parity import _batch_specs

pytestmark = pytest.mark.gpu


def _batched(precision=capi.FP32):
    from starpolymersmd_gb300 import workloads as W
    return W.build(_batch_specs(), precision=precision)


def _state(ctx):
    out = []
    for r in range(ctx.n_rep):
        out += list(ctx.get_fluid(r)) + list(ctx.get_monomers(r))
        out.append(np.array([ctx.delrx(r), ctx.verlet_rebuilds(r)]))
    return out


def _assert_same(a, b, precision=capi.FP32):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        if precision == capi.FP32:
            np.testing.assert_array_equal(x, y)
        else:
            H.close64(x, y)


@pytest.mark.parametrize("precision", [capi.FP32, capi.FP64])
def test_batched_restart_continues_the_run(precision):
    a = _batched(precision)
    b = _batched(precision)
    try:
        a.ctx.cycles(2)
        blob = a.ctx.checkpoint()
        a.ctx.cycles(3)
        a.ctx.synchronize()
        # b is a different run until it loads a's checkpoint
        b.ctx.cycles(1)
        b.ctx.restore(blob)
        b.ctx.cycles(3)
        b.ctx.synchronize()
        a.ctx.raise_on_device_error()
        b.ctx.raise_on_device_error()
        _assert_same(_state(a.ctx), _state(b.ctx), precision)
        # FP64 reductions whose order follows the binning ranks: to round-off
        _assert_same([a.ctx.temperature_all(), a.ctx.molecule_observables_all()],
                     [b.ctx.temperature_all(), b.ctx.molecule_observables_all()], capi.FP64)
    finally:
        a.close()
        b.close()


def _periodic(precision):
    L = 14
    sol = system.star_solution(5, 4, 6, 0.5, 5.0, 1.0, (L, L, L), np.random.default_rng(21))
    rep = dict(L=(L, L, L), n_fluid=3 * L ** 3, n_mono=sol.n, mol0_size=sol.stars[0].n,
               kT=1.0, shear=0.3, h=0.1, md_dt=0.01, seed=5, potential=capi.POT_LJ126,
               r_cut=2.5, r_verlet=2.8, flags=capi.REPLICA_PERIODIC_MD)
    ctx = capi.Context([rep], precision=precision, rng=capi.RNG_PHILOX, step_update=10,
                       mono_bin=capi.MONOBIN_WRAPPED, delrx_mode=capi.DELRX_PHYSICAL,
                       strict_cells=0)
    ctx.init_solvent(0, seed=5, shear_profile=True)
    ctx.set_monomers(0, sol.pos, sol.vel, np.zeros_like(sol.pos), sol.mass, sol.amphi,
                     sol.anchor)
    ctx.set_bonds(0, sol.bond_src, sol.bond_dst)
    ctx.set_molecules(0, sol.mol_start)
    ctx.init_md()
    return ctx


@pytest.mark.parametrize("precision", [capi.FP32, capi.FP64])
def test_periodic_restart_through_a_file(tmp_path, precision):
    path = os.path.join(str(tmp_path), "run.smpc")
    with _periodic(precision) as a, _periodic(precision) as b:
        a.cycles(2)
        a.checkpoint_write(path)
        a.cycles(2)
        for t in range(1, 11):  # call by call after the restart as well
            a.md_substeps(1)
            a.mpc_step(t, 0.1)
        a.synchronize()
        b.checkpoint_read(path)
        b.cycles(2)
        for t in range(1, 11):
            b.md_substeps(1)
            b.mpc_step(t, 0.1)
        b.synchronize()
        a.raise_on_device_error()
        b.raise_on_device_error()
        _assert_same(_state(a), _state(b), precision)


def test_checkpoint_of_other_replicas_is_refused():
    a = _batched()
    try:
        with _periodic(capi.FP32) as p:
            p.cycles(1)
            before = _state(p)
            with pytest.raises(capi.SmpcError):
                p.restore(a.ctx.checkpoint())
            with pytest.raises(capi.SmpcError):
                p.restore(b"not a checkpoint" * 8)
            _assert_same(before, _state(p))
            p.cycles(1)  # still usable
            p.raise_on_device_error()
    finally:
        a.close()
