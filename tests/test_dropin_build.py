"""The reference-side binding: StarPolymersMD's own drivers compiled unchanged
against the GPU drop-ins (starpolymersmd_gb300/dropin: an MPC class with the
reference's interface over the C ABI, a Thermostat subclass, the shared
per-Box device context) and linked to libsmpc.

Runs where the reference checkout is available (it is not shipped); the
drivers are only built and inspected here, not run (they need a GPU and
write into ./results).
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "starpolymersmd_gb300", "dropin")
SHIM_INC = os.path.join(ROOT, "oracle", "refbuild", "shim", "inc")


def _reference():
    ref = os.environ.get("SMPC_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
    if not os.path.isdir(os.path.join(ref, "star-polymers", "src")):
        pytest.skip("reference checkout not available")
    return ref


def test_reference_drivers_build_against_dropins(tmp_path):
    ref = _reference()
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from starpolymersmd_gb300 import build as B
    lib = B.build()
    out = tmp_path / "bin"
    res = subprocess.run(
        ["make", "-C", DROPIN, f"REF={ref}", f"EIGEN={SHIM_INC}",
         f"SMPC={os.path.dirname(lib)}", f"OUT={out}", "all"],
        capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-4000:]
    for exe in ("star-polymers", "mpc-test"):
        path = out / exe
        assert path.exists()
        # the drivers call the C ABI (no CPU MPC linked in) ...
        und = subprocess.run(["nm", "-u", str(path)], capture_output=True, text=True).stdout
        for sym in ("smpc_create", "smpc_mpc_bin", "smpc_mpc_collide", "smpc_cell_counts",
                    "smpc_get_fluid", "smpc_cell_members", "smpc_temperature"):
            assert sym in und, (exe, sym)
        if exe == "star-polymers":
            # the MPC-off integrator (AndersenStochastic) steps on the device
            for sym in ("smpc_stage_andersen", "smpc_md_substeps"):
                assert sym in und, (exe, sym)
        # ... and resolve them from the in-tree libsmpc
        ldd = subprocess.run(["ldd", str(path)], capture_output=True, text=True).stdout
        assert os.path.realpath(lib) in ldd or os.path.basename(lib) in ldd


def test_call_sequence_program_builds(tmp_path):
    # tests/dropin_sequence.cpp (the drop-in's call sequence, run against the
    # reference's fixtures by the GPU tests) builds from include/smpc.h and
    # links to the in-tree libsmpc, calling what the drop-in calls
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from starpolymersmd_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "dropin_sequence")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "dropin_sequence.cpp"), "-L", libdir, "-lsmpc",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True, timeout=300)
    und = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    for sym in ("smpc_create", "smpc_set_fluid", "smpc_set_monomers", "smpc_set_bonds",
                "smpc_init_md", "smpc_md_substeps", "smpc_epot", "smpc_set_delrx", "smpc_mpc_bin",
                "smpc_cell_counts", "smpc_mpc_collide", "smpc_error_word", "smpc_get_fluid",
                "smpc_cell_members", "smpc_get_monomer_state_all", "smpc_temperature"):
        assert sym in und, sym
    order = subprocess.run([exe, "--shift-order"], capture_output=True, text=True, check=True)
    assert sorted(int(x) for x in order.stdout.split()) == [0, 1, 2]
