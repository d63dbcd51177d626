"""The C ABI library builds for sm_103a, loads, and exports every entry
point that include/openmoc_gb300.h declares (no GPU needed: nothing here
calls into the device)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "openmoc_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(moc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "moc_create" in names and "moc_transport_sweep" in names
    assert len(names) >= 40


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists(
    "/usr/local/cuda/bin/nvcc"), reason="CUDA toolkit absent")
def test_library_builds_and_exports_every_declared_symbol():
    from openmoc_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True,
                         text=True).stdout
    for n in declared_functions():
        assert re.search(rf"\bT {n}$", out, re.M), n


def test_python_binding_covers_the_header():
    from openmoc_gb300 import _native
    assert set(_native.exported_symbols()) == set(declared_functions())


def test_library_is_sm_103a_only():
    from openmoc_gb300 import build
    path = build.build()
    cuobj = shutil.which("cuobjdump") or "/usr/local/cuda/bin/cuobjdump"
    if not os.path.exists(cuobj):
        pytest.skip("cuobjdump absent")
    # list the embedded ELF images only (architecture names), no disassembly
    out = subprocess.run([cuobj, "--list-elf", path], capture_output=True,
                         text=True).stdout
    assert "sm_103a" in out
    for other in ("sm_90", "sm_100", "sm_80"):
        assert f".{other}." not in out
