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
        ("keff", C.c_double), ("leakage", C.c_void_p),
        ("stab_flux", C.c_void_p), ("stab_type", C.c_int32), ("stab_factor", C.c_double),
    ]


class _LSGeometry(C.Structure):
    _fields_ = [("seg_x", C.c_void_p), ("seg_y", C.c_void_p),
                ("ang_dir", C.c_void_p), ("ang_wgt", C.c_void_p),
                ("pol_sin", C.c_void_p), ("pol_wgt", C.c_void_p),
                ("seg_z", C.c_void_p), ("pol_cos", C.c_void_p)]


class _LSState(C.Structure):
    _fields_ = [("ilem", C.c_void_p), ("src_const", C.c_void_p),
                ("mom", C.c_void_p), ("red_xyz", C.c_void_p),
                ("fixed_xy", C.c_void_p), ("negative_allowed", C.c_int32),
                ("num_flat", C.c_int32), ("stab_xyz", C.c_void_p)]


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
        lib.oracle_sweep_currents.argtypes = [P, S, C.c_void_p, C.c_void_p, C.c_int,
                                              C.c_void_p]
        lib.oracle_add_source.argtypes = [P, S, C.c_int]
        lib.oracle_add_source.restype = C.c_long
        lib.oracle_compute_keff.argtypes = [P, S]
        lib.oracle_normalize.argtypes = [P, S]
        lib.oracle_normalize.restype = C.c_double
        lib.oracle_residual.argtypes = [P, S, C.c_int]
        lib.oracle_residual.restype = C.c_double
        lib.oracle_store.argtypes = [P, S]
        lib.oracle_compute_stabilizing_flux.argtypes = [P, S]
        lib.oracle_stabilize_flux.argtypes = [P, S]
        lib.oracle_flatten.argtypes = [P, S, C.c_double]
        lib.oracle_zero_track_fluxes.argtypes = [P, S]
        lib.oracle_real_size.restype = C.c_int
        LG, LS = C.POINTER(_LSGeometry), C.POINTER(_LSState)
        lib.oracle_ls_constants.argtypes = [P, LG, LS]
        lib.oracle_ls_constants.restype = C.c_int
        lib.oracle_ls_flatten.argtypes = [P, S, LS, C.c_double]
        lib.oracle_ls_normalize.argtypes = [P, S, LS]
        lib.oracle_ls_normalize.restype = C.c_double
        lib.oracle_ls_compute_sources.argtypes = [P, S, LS, C.c_int]
        lib.oracle_ls_compute_sources.restype = C.c_long
        lib.oracle_ls_sweep.argtypes = [P, LG, S, LS]
        lib.oracle_ls_add_source.argtypes = [P, S, LS]
        lib.oracle_ls_add_source.restype = C.c_long
        lib.oracle_ls_compute_eigenvalue.argtypes = [P, LG, S, LS, C.c_int, C.c_int,
                                                     C.c_double, C.POINTER(C.c_double)]
        lib.oracle_ls_compute_eigenvalue.restype = C.c_int
        lib.oracle_ls_compute_source.argtypes = [P, LG, S, LS, C.c_int, C.c_double,
                                                 C.c_int, C.c_double,
                                                 C.POINTER(C.c_double)]
        lib.oracle_ls_compute_source.restype = C.c_int
        lib.oracle_ls_compute_flux.argtypes = [P, LG, S, LS, C.c_int, C.c_double,
                                               C.POINTER(C.c_double)]
        lib.oracle_ls_compute_flux.restype = C.c_int
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
        self.leakage = None
        self._cs = _State(_ptr(self.phi), _ptr(self.phi_old), _ptr(self.reduced),
                          _ptr(self.fixed), _ptr(self.boundary), _ptr(self.start), 1.0,
                          None, None, 0, 0.0)
        self.stab_flux = None
        self.num_iterations = 0
        self.residual = 0.0

    def set_keff_from_neutron_balance(self) -> None:
        """keff = fission / (absorption + leakage), the leakage tallied per
        track at vacuum ends (Solver::setKeffFromNeutronBalance)."""
        self.leakage = np.zeros(self.p.num_tracks, self.real)
        self._cs.leakage = _ptr(self.leakage)

    def stabilize_transport(self, factor: float, kind: int) -> None:
        """Solver::stabilizeTransport: kind 0 DIAGONAL, 1 YAMAMOTO, 2 GLOBAL."""
        self.stab_flux = np.zeros(self.p.num_fsrs * self.p.num_groups, self.real)
        self._cs.stab_flux = _ptr(self.stab_flux)
        self._cs.stab_type = int(kind)
        self._cs.stab_factor = float(factor)

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

    def sweep_currents(self, cell: np.ndarray, end_face: np.ndarray, nx: int,
                       cur: np.ndarray) -> None:
        """The sweep with CMFD partial currents added into cur [cells][4][G]
        (FP64)."""
        assert cell.dtype == np.int32 and end_face.dtype == np.int8
        assert cur.dtype == np.float64 and cur.flags.c_contiguous
        self.lib.oracle_sweep_currents(C.byref(self._cp), C.byref(self._cs),
                                       _ptr(cell), _ptr(end_face), nx, _ptr(cur))

    def flatten(self, value: float = 1.0) -> None:
        self.lib.oracle_flatten(C.byref(self._cp), C.byref(self._cs), value)

    def zero_track_fluxes(self) -> None:
        self.lib.oracle_zero_track_fluxes(C.byref(self._cp), C.byref(self._cs))

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

    def compute_stabilizing_flux(self) -> None:
        self.lib.oracle_compute_stabilizing_flux(C.byref(self._cp), C.byref(self._cs))

    def stabilize_flux(self) -> None:
        self.lib.oracle_stabilize_flux(C.byref(self._cp), C.byref(self._cs))

    def configure(self, scalars) -> None:
        """The solver options a fixture was made with: keff from the neutron
        balance, transport stabilization."""
        if int(scalars.get("keff_balance", 0)):
            self.set_keff_from_neutron_balance()
        if int(scalars.get("stab_type", -1)) >= 0:
            self.stabilize_transport(scalars["stab_factor"], int(scalars["stab_type"]))


class LSOracle(Oracle):
    """The linear-source CPU solver (CPULSSolver, 2D or explicit 3D) over one
    packed problem plus its linear-source geometry: ``ls`` maps seg_x,
    seg_y, ang_dir, ang_wgt, pol_sin, pol_wgt (the arrays of
    include/openmoc_gb300.h's moc_ls_geometry), in 3D also seg_z and
    pol_cos, and optionally fixed_xy ([R][2][G] fixed source moments, 2D).
    The expansion inverse and source constants have NC = 3 coefficients in
    2D, 6 in 3D."""

    def __init__(self, problem, ls, precision: str = "f32", num_threads: int = 0,
                 negative_fluxes_allowed: bool = False):
        super().__init__(problem, precision, num_threads)
        R, G = problem.num_fsrs, problem.num_groups
        self.geo_arrays = {
            "seg_x": np.ascontiguousarray(ls["seg_x"], np.float32),
            "seg_y": np.ascontiguousarray(ls["seg_y"], np.float32),
            "ang_dir": np.ascontiguousarray(ls["ang_dir"], np.float64),
            "ang_wgt": np.ascontiguousarray(ls["ang_wgt"], np.float64),
            "pol_sin": np.ascontiguousarray(ls["pol_sin"], np.float64),
            "pol_wgt": np.ascontiguousarray(ls["pol_wgt"], np.float64),
        }
        self.nc = 3
        if getattr(problem, "solve_3d", 0):
            self.nc = 6
            self.geo_arrays["seg_z"] = np.ascontiguousarray(ls["seg_z"], np.float32)
            self.geo_arrays["pol_cos"] = np.ascontiguousarray(ls["pol_cos"], np.float64)
        g = self.geo_arrays
        self._cg = _LSGeometry(_ptr(g["seg_x"]), _ptr(g["seg_y"]), _ptr(g["ang_dir"]),
                               _ptr(g["ang_wgt"]), _ptr(g["pol_sin"]),
                               _ptr(g["pol_wgt"]), _ptr(g.get("seg_z")),
                               _ptr(g.get("pol_cos")))
        self.ilem = np.zeros(R * self.nc, np.float64)
        self.src_const = np.zeros(R * self.nc * G, self.real)
        self.mom = np.zeros(R * 3 * G, self.real)
        self.red_xyz = np.zeros(R * 3 * G, self.real)
        fx = ls.get("fixed_xy")
        self.fixed_xy = None if fx is None else np.ascontiguousarray(fx, self.real)
        self._cl = _LSState(_ptr(self.ilem), _ptr(self.src_const), _ptr(self.mom),
                            _ptr(self.red_xyz), _ptr(self.fixed_xy),
                            1 if negative_fluxes_allowed else 0, 0)

    def stabilize_transport(self, factor: float, kind: int) -> None:
        """Solver::stabilizeTransport on CPULSSolver, which stabilizes the
        flux moments too (_stabilize_moments is set in its constructor,
        src/CPULSSolver.cpp:19)."""
        super().stabilize_transport(factor, kind)
        self.stab_xyz = np.zeros(self.p.num_fsrs * 3 * self.p.num_groups, self.real)
        self._cl.stab_xyz = _ptr(self.stab_xyz)

    def constants(self) -> int:
        return self.lib.oracle_ls_constants(C.byref(self._cp), C.byref(self._cg),
                                            C.byref(self._cl))

    def compute_eigenvalue(self, max_iters=1000, res_type=FISSION_SOURCE, tol=1e-5):
        r = C.c_double()
        self.num_iterations = self.lib.oracle_ls_compute_eigenvalue(
            C.byref(self._cp), C.byref(self._cg), C.byref(self._cs), C.byref(self._cl),
            max_iters, res_type, tol, C.byref(r))
        self.residual = r.value
        return self.num_iterations

    def compute_source(self, max_iters=1000, k_eff=1.0, res_type=TOTAL_SOURCE, tol=1e-5):
        r = C.c_double()
        self.num_iterations = self.lib.oracle_ls_compute_source(
            C.byref(self._cp), C.byref(self._cg), C.byref(self._cs), C.byref(self._cl),
            max_iters, k_eff, res_type, tol, C.byref(r))
        self.residual = r.value
        return self.num_iterations

    def compute_flux(self, max_iters=1000, tol=1e-5):
        r = C.c_double()
        self.num_iterations = self.lib.oracle_ls_compute_flux(
            C.byref(self._cp), C.byref(self._cg), C.byref(self._cs), C.byref(self._cl),
            max_iters, tol, C.byref(r))
        self.residual = r.value
        return self.num_iterations

    def compute_sources(self, iteration: int) -> int:
        return self.lib.oracle_ls_compute_sources(C.byref(self._cp), C.byref(self._cs),
                                                  C.byref(self._cl), iteration)

    def sweep(self) -> None:
        self.lib.oracle_ls_sweep(C.byref(self._cp), C.byref(self._cg), C.byref(self._cs),
                                 C.byref(self._cl))

    def add_source(self) -> int:
        return self.lib.oracle_ls_add_source(C.byref(self._cp), C.byref(self._cs),
                                             C.byref(self._cl))

    def normalize(self) -> float:
        return self.lib.oracle_ls_normalize(C.byref(self._cp), C.byref(self._cs),
                                            C.byref(self._cl))
