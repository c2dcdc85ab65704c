"""The drop-in MPC's call sequence through the C ABI, from C++.

tests/dropin_sequence.cpp makes the calls starpolymersmd_gb300/dropin/
(MPC_gpu.cpp, smpc_box.cpp) makes, in the same order and with the same host
logic, and sees only include/smpc.h and libsmpc.so; the drop-in sources
themselves compile only inside a reference checkout. It is compiled here with
g++, fed a reference fixture's initial state and the reference's Rand stream
(rebuilt from the fixture's recorded draws in the reference's draw order:
three grid-shift uniforms, then per cell a gamma variate when it holds two or
more particles, then phi and theta), and its results are compared with the
reference's at the FP64 tolerance: the Lees-Edwards offset bit for bit,
occupancies and cell memberships exactly, states, energies and temperature to
1e-12, and the kinetic energy and filled cells of the host cell-list mirror
the drop-in's per-cell getters read.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from starpolymersmd_gb300 import capi
from tests import golden_replay as gr
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TAG = 0x5350


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    capi.load()  # the library must have been built
    libdir = os.path.dirname(capi.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_sequence")
    # -ffp-contract=off as in the drop-in's Makefile: g++ on aarch64 would
    # otherwise fuse the delrx advance into an FMA and round it differently
    # from the reference built on x86
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "dropin_sequence.cpp"), "-L", libdir, "-lsmpc",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    return exe


def shift_order(exe):
    out = subprocess.run([exe, "--shift-order"], check=True, capture_output=True, text=True)
    return [int(x) for x in out.stdout.split()]


def rand_tape(fx, order):
    """The reference's Rand values of every collision in draw order."""
    tape = []
    for k in range(len(fx["coll_steps"])):
        shift = fx["shift"][k]
        u = shift + 0.5
        # the reference formed shift = u - 0.5; u - 0.5 gives the same bits back
        assert np.array_equal(u - 0.5, shift)
        for j in range(3):
            tape.append(u[order.index(j)])
        tot = fx["count_total"][k]
        for c in range(len(tot)):
            if tot[c] >= 2:
                tape.append(fx["gamma"][k][c])
            tape.append(fx["u_phi"][k][c])
            tape.append(fx["u_theta"][k][c])
    return np.array(tape, dtype=np.float64)


def write_input(path, fx, tape):
    n = len(fx["fluid_pos0"])
    m = len(fx["mono_pos0"])
    b = len(fx["bond_src"])
    L = [int(x) for x in fx["L"]]
    with open(path, "wb") as f:
        f.write(struct.pack("=11i", *L, n, m, b, int(fx["n_loop"]), int(fx["step_update"]),
                            int(fx["with_md"]), len(tape), TAG))
        f.write(struct.pack("=7d", float(fx["kT"]), float(fx["shear"]), float(fx["h"]),
                            float(fx["md_dt"]), float(fx["lam"]), 1.5, 2.0))
        for key, dt in (("fluid_pos0", np.float64), ("fluid_vel0", np.float64),
                        ("mono_pos0", np.float64), ("mono_vel0", np.float64),
                        ("mono_force0", np.float64), ("mono_mass", np.float64),
                        ("mono_amphi", np.int32), ("mono_anchor", np.int32),
                        ("bond_src", np.int32), ("bond_dst", np.int32)):
            f.write(np.ascontiguousarray(fx[key], dtype=dt).tobytes())
        f.write(tape.tobytes())


def mirror_ekin(fcell, fvel, mcell, mvel, mass, n_cells):
    """MPC::calculateEkinTotal over cell lists of solvent (mass 1) and monomers."""
    msum = np.bincount(fcell, minlength=n_cells).astype(np.float64)
    p = np.stack([np.bincount(fcell, weights=fvel[:, d], minlength=n_cells) for d in range(3)], 1)
    ok = mcell >= 0
    msum += np.bincount(mcell[ok], weights=mass[ok], minlength=n_cells)
    for d in range(3):
        p[:, d] += np.bincount(mcell[ok], weights=mass[ok] * mvel[ok, d], minlength=n_cells)
    cmv = np.divide(p, msum[:, None], out=np.zeros_like(p), where=msum[:, None] > 0)
    return 0.5 * float(((fvel - cmv[fcell]) ** 2).sum())


@pytest.mark.parametrize("name", ["star_mpc_L12"])
def test_dropin_call_sequence_replays_reference(program, golden_dir, tmp_path, name):
    fx = gr.load(os.path.join(golden_dir, name + ".npz"))
    order = shift_order(program)
    assert sorted(order) == [0, 1, 2]
    tape = rand_tape(fx, order)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, fx, tape)
    run = subprocess.run([program, inp, outp], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, (run.returncode, run.stdout[-2000:], run.stderr[-2000:])
    out = np.fromfile(outp, dtype=np.float64)

    n, m = len(fx["fluid_pos0"]), len(fx["mono_pos0"])
    n_cells = int(np.prod(fx["L"]))
    coll = gr.collision_index(fx)
    su = int(fx["step_update"])
    at = 0

    def take(k):
        nonlocal at
        v = out[at: at + k]
        assert len(v) == k, "output too short"
        at += k
        return v

    for t in range(int(fx["n_loop"])):
        delrx_host, delrx_dev, epot = take(3)
        assert delrx_host == fx["delrx"][t]
        H.close64(epot, fx["epot"][t])
        pos, vel, force = (take(3 * m).reshape(m, 3) for _ in range(3))
        H.close64(pos, fx["mono_pos"][t])
        H.close64(vel, fx["mono_vel"][t])
        H.close64(force, fx["mono_force"][t], rtol=1e-11)
        k = coll.get(t)
        assert (k is not None) == (t % su == 0)
        if k is None:
            continue
        assert delrx_dev == delrx_host
        np.testing.assert_array_equal(take(n_cells), fx["count_total"][k])
        H.close64(take(3 * n).reshape(n, 3), fx["fluid_pos"][k])
        fvel = take(3 * n).reshape(n, 3)
        H.close64(fvel, fx["fluid_vel"][k])
        fcell = take(n).astype(np.int64)
        mcell = take(m).astype(np.int64)
        np.testing.assert_array_equal(fcell, fx["fluid_cell"][k])
        np.testing.assert_array_equal(mcell, fx["mono_cell"][k])
        T, ekin, filled = take(3)
        H.close64(T, fx["temperature"][k])
        want = mirror_ekin(fx["fluid_cell"][k], fx["fluid_vel"][k], fx["mono_cell"][k],
                           fx["mono_vel"][t], fx["mono_mass"], n_cells)
        np.testing.assert_allclose(ekin, want, rtol=1e-12)
        assert filled == int((fx["count_fluid"][k] > 0).sum())
    (taken,) = take(1)
    assert at == len(out)
    assert int(taken) == len(tape)
