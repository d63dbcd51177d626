"""The FP64 host coarse solve of the CUDA library's CMFD
(openmoc_gb300/csrc/cmfd_solve.cpp, compiled here with a small C shim,
tests/cmfd_host/shim.cpp) against the CMFD oracle, step by step on
OpenMOC's CMFD fixtures, without a GPU: the same tallies in, the same
coarse eigenvalue and prolongation ratios out."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import CMFD_CASES, ROOT, load_case
from oracle.oracle import Oracle
from test_oracle_cmfd import cmfd_oracle_for

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int32)


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cmfd") / "libcmfdshim.so")
    subprocess.check_call([
        "g++", "-O2", "-std=c++17", "-shared", "-fPIC",
        "-I", os.path.join(ROOT, "include"),
        os.path.join(ROOT, "tests", "cmfd_host", "shim.cpp"),
        os.path.join(ROOT, "openmoc_gb300", "csrc", "cmfd_solve.cpp"),
        "-o", out])
    lib = C.CDLL(out)
    lib.shim_create.restype = C.c_void_p
    lib.shim_create.argtypes = [C.c_int, C.c_int, D, D, C.c_int, C.c_int, I, I,
                                C.c_int, D, D, C.c_double, C.c_double, C.c_int,
                                C.c_int]
    lib.shim_set_fine.argtypes = [C.c_void_p, C.c_int, D, D, D, D, C.c_int, I, I, D]
    lib.shim_reset.argtypes = [C.c_void_p, C.c_double]
    lib.shim_set_source_threshold.argtypes = [C.c_void_p, C.c_double]
    lib.shim_step.restype = C.c_double
    lib.shim_step.argtypes = [C.c_void_p, C.c_int, D, C.POINTER(C.c_float), C.c_int,
                              D, C.POINTER(C.c_int)]
    lib.shim_destroy.argtypes = [C.c_void_p]
    return lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


@pytest.mark.parametrize("case", ["cmfd_lat3", "cmfd_lat5_vac"])
def test_host_coarse_solve_matches_oracle(shim, case):
    p, sc, _ = load_case(case, "f64")
    cm = cmfd_oracle_for(p, CMFD_CASES[case])
    o = Oracle(p, "f64", num_threads=8)
    G, M, R = p.num_groups, p.num_materials, p.num_fsrs
    # (cell, material) pairs in cell-major order, as the library makes them
    cell, mat, vol = cm.cell, p.fsr_mat, p.fsr_vol.astype(np.float64)
    keys = sorted({(int(c), int(m)) for c, m in zip(cell, mat)})
    pid = {k: i for i, k in enumerate(keys)}
    fsr_pair = np.array([pid[(int(c), int(m))] for c, m in zip(cell, mat)])
    pair_cell = np.array([k[0] for k in keys], np.int32)
    pair_mat = np.array([k[1] for k in keys], np.int32)
    cell_vol = np.zeros(cm.C)
    np.add.at(cell_vol, cell, vol)
    wx, wy = np.ascontiguousarray(cm.wx), np.ascontiguousarray(cm.wy)
    go = np.ascontiguousarray(cm.group_of, np.int32)
    bc = np.array(cm.bc, np.int32)
    h = shim.shim_create(cm.nx, cm.ny, _p(wx, C.c_double), _p(wy, C.c_double), G,
                         cm.E, _p(go, C.c_int32), _p(bc, C.c_int32), cm.edc_mu.size,
                         _p(cm.edc_mu, C.c_double), _p(cm.edc_w, C.c_double),
                         cm.relaxation, cm.sor, 1, 0)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (cm.st, cm.nf, cm.chi, cm.ss)]
    shim.shim_set_fine(h, M, *[_p(a, C.c_double) for a in arrs], len(keys),
                       _p(pair_cell, C.c_int32), _p(pair_mat, C.c_int32),
                       _p(cell_vol, C.c_double))
    tol = sc["tolerance"]
    shim.shim_reset(h, tol)
    cm.reset(tol)
    o.keff = 1.0
    o.zero_track_fluxes()
    o.flatten(1.0)
    o.normalize()
    o.store()
    cur = np.zeros((cm.C, 4, G))
    ratio = np.zeros(cm.C * cm.E)
    pw = C.c_int()
    for i in range(8):
        o.compute_sources(i)
        cur[:] = 0.0
        o.sweep_currents(cm.cell, cm.end_face, cm.nx, cur)
        o.add_source()
        phi = o.phi.reshape(R, G).astype(np.float64)
        cur32 = np.ascontiguousarray(cur, np.float32)        # the device tallies FP32
        k_o, r_o = cm.compute_keff(i, phi, cur32.astype(np.float64))
        S = np.zeros((len(keys), G))
        np.add.at(S, fsr_pair, phi * vol[:, None])
        S = np.ascontiguousarray(S)
        k_s = shim.shim_step(h, i, _p(S, C.c_double), _p(cur32, C.c_float), G,
                             _p(ratio, C.c_double), C.byref(pw))
        assert abs(k_s - k_o) < 1e-9 * abs(k_o), (i, k_s, k_o)
        assert pw.value == cm.power_iterations, i
        np.testing.assert_allclose(ratio.reshape(cm.C, cm.E), r_o, rtol=1e-7,
                                   atol=1e-12)
        o.keff = k_o
        o.phi[:] = (phi * cm.update_ratios(i, r_o)[:, cm.group_of]).ravel()
        o.normalize()
        res = o.residual_of(1)
        cm.source_threshold = 0.01 * (res if res > 0 else 1e-6)
        shim.shim_set_source_threshold(h, cm.source_threshold)
        o.store()
    shim.shim_destroy(h)
