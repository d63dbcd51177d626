"""The OpenMOC-side drop-in (openmoc_gb300/adapter/GB300Solver.{h,cpp})
compiles against OpenMOC's own headers, links with OpenMOC's library and
libopenmoc_gb300.so, and runs through OpenMOC's API.  Needs OpenMOC's source
tree (it is the reference project itself), named by the environment variable
OPENMOC_SOURCE, so it is skipped where that is unset; without a GPU the
driver reports the adapter's error instead of a result, which must be the
ERROR-level exception OpenMOC raises."""
import os
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("OPENMOC_SOURCE", "")


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "src")),
                    reason="set OPENMOC_SOURCE to an OpenMOC source tree to build the "
                           "adapter against it")
def test_adapter_builds_and_runs(tmp_path):
    from openmoc_gb300 import build
    lib = build.build()
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"),
                           f"REF={REF}", f"OUT={os.path.join(ROOT, 'oracle', '_ref')}",
                           f"-j{os.cpu_count() or 4}"], cwd=ROOT)
    exe = str(tmp_path / "adapter_driver")
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-O2", "-fopenmp", "-std=c++11", "-w", "-DGCC", "-DOPENMP",
           "-DVEC_ALIGNMENT=64", "-DFP_PRECISION=float", "-DSINGLE", "-DVEC_LENGTH=8",
           "-DCMFD_PRECISION=float", "-DLINALG_TOL=1E-7",
           "-I", os.path.join(REF, "src"),
           "-I", os.path.join(ROOT, "openmoc_gb300", "adapter"),
           os.path.join(ROOT, "tests", "adapter", "adapter_driver.cpp"),
           os.path.join(ROOT, "openmoc_gb300", "adapter", "GB300Solver.cpp"),
           os.path.join(ROOT, "oracle", "_ref", "libopenmoc_f32.a"),
           lib, f"-Wl,-rpath,{os.path.dirname(lib)}",
           f"-L{cuda}/lib64", "-lcudart", f"-Wl,-rpath,{cuda}/lib64", "-o", exe]
    subprocess.check_call(cmd)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    assert lines[0].startswith("cpu keff")
    gpu = [l for l in lines if l.startswith("gb300")]
    assert gpu, out.stdout
    if gpu[0].startswith("gb300 error"):
        # no usable GPU here: the C ABI error surfaced as OpenMOC's ERROR
        assert "moc_create failed" in gpu[0]
    else:
        k_cpu = float(lines[0].split()[2])
        k_gpu = float(gpu[0].split()[2])
        assert abs(k_cpu - k_gpu) < 1e-5
    ls = [l for l in lines if l.startswith("gb300 ls")]
    assert ls, out.stdout
    if ls[0].startswith("gb300 ls error"):
        assert "moc_create failed" in ls[0]
