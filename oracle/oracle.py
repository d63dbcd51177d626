"""ctypes front end of the C oracle (oracle/moc_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
baseline.  Nothing in the product package imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

SCALAR_FLUX, FISSION_SOURCE, TOTAL_SOURCE = 0, 1, 2


class _Problem(C.Structure):
    _fields_ = [
        ("num_groups", C.c_int32), ("num_polar_half", C.c_int32),
        ("num_angles", C.c_int32), ("num_materials", C.c_int32),
        ("num_fsrs", C.c_int64), ("num_tracks", C.c_int64),
        ("num_segments", C.c_int64),
        ("seg_len", C.c_void_p), ("seg_fsr", C.c_void_p),
        ("seg_off", C.c_void_p), ("track_ang", C.c_void_p),
        ("next", C.c_void_p), ("flags", C.c_void_p),
        ("weights", C.c_void_p), ("inv_sin", C.c_void_p),
        ("sigma_t", C.c_void_p), ("sigma_s", C.c_void_p),
        ("nu_sigma_f", C.c_void_p), ("chi", C.c_void_p),
        ("fsr_mat", C.c_void_p), ("fsr_vol", C.c_void_p),
        ("solve_3d", C.c_int32), ("num_threads", C.c_int32),
    ]


class _State(C.Structure):
    _fields_ = [
        ("phi", C.c_void_p), ("phi_old", C.c_void_p), ("reduced", C.c_void_p),
        ("fixed", C.c_void_p), ("boundary", C.c_void_p), ("start", C.c_void_p),
        ("keff", C.c_double),
    ]


def build() -> None:
    subprocess.check_call(["bash", os.path.join(HERE, "build.sh")])


_LIBS = {}


def _lib(precision: str):
    if precision not in _LIBS:
        path = os.path.join(BUILD, f"libmoc_oracle_{precision}.so")
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        P, S = C.POINTER(_Problem), C.POINTER(_State)
        lib.oracle_compute_eigenvalue.argtypes = [P, S, C.c_int, C.c_int, C.c_double,
                                                  C.POINTER(C.c_double)]
        lib.oracle_compute_eigenvalue.restype = C.c_int
        lib.oracle_compute_source.argtypes = [P, S, C.c_int, C.c_double, C.c_int,
                                              C.c_double, C.POINTER(C.c_double)]
        lib.oracle_compute_source.restype = C.c_int
        lib.oracle_compute_flux.argtypes = [P, S, C.c_int, C.c_double,
                                            C.POINTER(C.c_double)]
        lib.oracle_compute_flux.restype = C.c_int
        lib.oracle_compute_sources.argtypes = [P, S, C.c_int, C.c_int]
        lib.oracle_compute_sources.restype = C.c_long
        lib.oracle_sweep.argtypes = [P, S]
        lib.oracle_add_source.argtypes = [P, S, C.c_int]
        lib.oracle_add_source.restype = C.c_long
        lib.oracle_compute_keff.argtypes = [P, S]
        lib.oracle_normalize.argtypes = [P, S]
        lib.oracle_normalize.restype = C.c_double
        lib.oracle_residual.argtypes = [P, S, C.c_int]
        lib.oracle_residual.restype = C.c_double
        lib.oracle_store.argtypes = [P, S]
        lib.oracle_flatten.argtypes = [P, S, C.c_double]
        lib.oracle_zero_track_fluxes.argtypes = [P, S]
        lib.oracle_real_size.restype = C.c_int
        _LIBS[precision] = lib
    return _LIBS[precision]


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


class Oracle:
    """CPU solver state over one packed problem (float or double)."""

    def __init__(self, problem, precision: str = "f32", num_threads: int = 0):
        self.lib = _lib(precision)
        self.p = problem.contiguous()
        self.real = np.float32 if precision == "f32" else np.float64
        R, G = problem.num_fsrs, problem.num_groups
        nb = 2 * problem.num_tracks * problem.fluxes_per_track
        self.phi = np.zeros(R * G, self.real)
        self.phi_old = np.zeros(R * G, self.real)
        self.reduced = np.zeros(R * G, self.real)
        self.fixed = (None if problem.fixed_sources is None
                      else np.ascontiguousarray(problem.fixed_sources, self.real))
        self.boundary = np.zeros(nb, np.float32)
        self.start = np.zeros(nb, np.float32)
        pp = self.p
        self._cp = _Problem(
            pp.num_groups, pp.num_polar_half, pp.num_angles, pp.num_materials,
            pp.num_fsrs, pp.num_tracks, pp.num_segments,
            _ptr(pp.seg_len), _ptr(pp.seg_fsr), _ptr(pp.seg_off), _ptr(pp.track_ang),
            _ptr(pp.next), _ptr(pp.flags), _ptr(pp.weights), _ptr(pp.inv_sin),
            _ptr(pp.sigma_t), _ptr(pp.sigma_s), _ptr(pp.nu_sigma_f), _ptr(pp.chi),
            _ptr(pp.fsr_mat), _ptr(pp.fsr_vol), pp.solve_3d, num_threads)
        self._cs = _State(_ptr(self.phi), _ptr(self.phi_old), _ptr(self.reduced),
                          _ptr(self.fixed), _ptr(self.boundary), _ptr(self.start), 1.0)
        self.num_iterations = 0
        self.residual = 0.0

    @property
    def keff(self) -> float:
        return self._cs.keff

    @keff.setter
    def keff(self, v: float) -> None:
        self._cs.keff = v

    def compute_eigenvalue(self, max_iters=1000, res_type=FISSION_SOURCE, tol=1e-5):
        r = C.c_double()
        self.num_iterations = self.lib.oracle_compute_eigenvalue(
            C.byref(self._cp), C.byref(self._cs), max_iters, res_type, tol, C.byref(r))
        self.residual = r.value
        return self.num_iterations

    def compute_source(self, max_iters=1000, k_eff=1.0, res_type=TOTAL_SOURCE, tol=1e-5):
        r = C.c_double()
        self.num_iterations = self.lib.oracle_compute_source(
            C.byref(self._cp), C.byref(self._cs), max_iters, k_eff, res_type, tol,
            C.byref(r))
        self.residual = r.value
        return self.num_iterations

    def compute_flux(self, max_iters=1000, tol=1e-5):
        r = C.c_double()
        self.num_iterations = self.lib.oracle_compute_flux(
            C.byref(self._cp), C.byref(self._cs), max_iters, tol, C.byref(r))
        self.residual = r.value
        return self.num_iterations

    # hook-level calls, mirroring the protected Solver hooks
    def compute_sources(self, iteration: int) -> int:
        return self.lib.oracle_compute_sources(C.byref(self._cp), C.byref(self._cs),
                                               iteration, 0)

    def sweep(self) -> None:
        self.lib.oracle_sweep(C.byref(self._cp), C.byref(self._cs))

    def add_source(self) -> int:
        return self.lib.oracle_add_source(C.byref(self._cp), C.byref(self._cs), 0)

    def compute_keff(self) -> None:
        self.lib.oracle_compute_keff(C.byref(self._cp), C.byref(self._cs))

    def normalize(self) -> float:
        return self.lib.oracle_normalize(C.byref(self._cp), C.byref(self._cs))

    def residual_of(self, res_type: int) -> float:
        return self.lib.oracle_residual(C.byref(self._cp), C.byref(self._cs), res_type)

    def store(self) -> None:
        self.lib.oracle_store(C.byref(self._cp), C.byref(self._cs))
