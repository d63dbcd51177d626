"""The C ABI library builds for sm_103a, loads, and exports every entry
point that the headers under include/ declare (no GPU needed: nothing here
calls into the device)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")
HEADER = os.path.join(INCLUDE, "openmoc_gb300.h")


def declared_functions(header=None):
    """Entry points declared by one header, or by every header."""
    paths = [header] if header else [os.path.join(INCLUDE, f)
                                     for f in sorted(os.listdir(INCLUDE))
                                     if f.endswith(".h")]
    names = set()
    for path in paths:
        text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
        names.update(re.findall(r"\b(moc_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions(HEADER)
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
    assert set(_native.exported_symbols()) == set(declared_functions(HEADER))


def test_python_binding_covers_the_server_header():
    from openmoc_gb300 import serving
    header = os.path.join(INCLUDE, "openmoc_gb300_serve.h")
    assert set(serving.exported_symbols()) == set(declared_functions(header))


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
