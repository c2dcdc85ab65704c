"""Host-side checks of the C ABI (no GPU needed): the in-tree library loads
and exports every entry point include/*.h declares, and the Python binding
binds exactly that set."""
import glob
import os
import re
import subprocess

import pytest

from starpolymersmd_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(smpc_\w+)\s*\(", text, flags=re.M))
    return names


@pytest.fixture(scope="module")
def lib_path():
    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (smpc_\w+)", out))
    decl = declared_symbols()
    assert decl, "no declarations found"
    assert decl <= exported, decl - exported


def test_binding_covers_the_header(lib_path):
    assert set(capi.EXPORTS) == declared_symbols()
    lib = capi.load(lib_path)
    for name in capi.EXPORTS:
        assert getattr(lib, name).restype is not None or name == "smpc_destroy"


def test_library_is_sm103a_only(lib_path):
    # the build passes exactly one -gencode: compute_103a -> sm_103a
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]

