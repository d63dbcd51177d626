"""Builds libopenmoc_gb300.so, the sm_103a CUDA library behind the C ABI of
``include/openmoc_gb300.h``.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` and linked into one shared
library in ``openmoc_gb300/_lib/``.  Nothing is installed outside the
source tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libopenmoc_gb300.so")

SOURCES = ["sweep.cu", "solver_kernels.cu", "moc_api.cu", "lattice.cpp",
           "noalloc.cu", "serve.cu", "sources_tc.cu", "linear_source.cu",
           "lattice_gpu.cu", "otf_sweep.cu", "cmfd.cu", "cmfd_solve.cpp"] + [
    f"sweep_p{ph}_e{e}.cu" for ph in (1, 2, 3) for e in (0, 1)] + [
    f"ls_sweep_p{ph}.cu" for ph in (1, 2, 3)]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build "
                       "libopenmoc_gb300.so")


def _flags(ptxas_verbose: bool):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                "-I", os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]
    if ptxas_verbose:
        f += ["-Xptxas", "-v"]
    # extra nvcc flags (e.g. -DMOC_SWEEP_MIN_BLOCKS=6) for tuning builds
    f += os.environ.get("MOC_NVCC_FLAGS", "").split()
    return f


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC)
                    if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "openmoc_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_verbose: bool = False, force: bool = False) -> str:
    """Compiles (if stale) and returns the path of libopenmoc_gb300.so."""
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    objs = []
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, os.path.splitext(s)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            extra = ["-Xcompiler", "-fopenmp"] if s.endswith(".cpp") else []
            # the lattice ray tracer gives the same segments on the host and
            # on the GPU, on x86 and Arm: no contraction of a*b+c into FMA
            if s in ("lattice.cpp", "lattice_gpu.cu"):
                extra += ["-Xcompiler", "-ffp-contract=off", "-fmad=false"]
            jobs.append([cc] + _flags(ptxas_verbose) + extra + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose or ptxas_verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lgomp"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv, force="-f" in sys.argv))
