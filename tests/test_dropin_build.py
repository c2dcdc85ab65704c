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
