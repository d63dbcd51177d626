"""Host-side mirror of OpenMOC's ``Solver`` interface over the GB300 C ABI.

:class:`GB300Solver` exposes the names, argument meanings and error
behaviour of ``openmoc.Solver`` (``src/Solver.h:433-585``): construct it,
give it tracks with :meth:`setTrackGenerator`, then call
:meth:`computeEigenvalue`, :meth:`computeSource` or :meth:`computeFlux`
and read :meth:`getKeff`, :meth:`getFlux`, :meth:`getNumIterations`.
Errors raise ``RuntimeError`` (:class:`openmoc_gb300._native.MOCError`), as
OpenMOC's SWIG layer turns ``log_printf(ERROR, ...)`` into RuntimeError
(``openmoc/swig/openmoc.i:106``).

"Track generator" here is a :class:`openmoc_gb300.problem.Problem`: the
packed tracks, segments, quadrature and cross sections that OpenMOC's
``TrackGenerator`` / ``Geometry`` hold (packed from OpenMOC objects by
``openmoc_gb300/adapter/pack_reference.h``, or produced by
:mod:`openmoc_gb300.lattice`).

Every solve runs on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import time
from typing import Optional

import numpy as np

from . import _native
from .problem import Problem

# residualType values of src/Solver.h:82-92
SCALAR_FLUX = 0
FISSION_SOURCE = 1
TOTAL_SOURCE = 2

EXP_TABLE = 0
EXP_INTRINSIC = 1


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class GB300Solver:
    """GB300 method-of-characteristics solver with OpenMOC's Solver API."""

    def __init__(self, track_generator: Optional[Problem] = None, device: int = 0):
        self._lib = _native.lib()
        self._ctx = None
        self._device = device
        self._problem: Optional[Problem] = None
        self._threshold = 1e-5
        self._exp_kind = None   # None: chosen by the autotuner
        self._fixed: dict = {}
        self._fixed_by_material: dict = {}
        self._num_iterations = 0
        self._total_time = 0.0
        self._keff = 1.0
        self._shape = None
        self._source_kind = "auto"
        self._negative_ok = False
        self._keff_balance = False
        self._stabilization = None
        self._instances = 0
        self._formation = "explicit"
        self._cmfd = None
        self._cmfd_keep = None
        if track_generator is not None:
            self.setTrackGenerator(track_generator)

    # ------------------------------------------------------------ lifetime
    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def close(self) -> None:
        if self._ctx is not None:
            self._lib.moc_destroy(self._ctx)
            self._ctx = None

    def _call(self, name: str, *args):
        _native.check(getattr(self._lib, name)(self._ctx, *args))

    def _need_ctx(self):
        if self._ctx is None:
            raise RuntimeError("The Solver is unable to compute since it does "
                               "not contain a TrackGenerator")

    # ---------------------------------------------------------- set up
    def setTrackGenerator(self, track_generator: Problem) -> None:
        """Uploads the packed tracks, quadrature, materials and FSRs
        (Solver::setTrackGenerator, src/Solver.cpp:412-454)."""
        p = track_generator
        if not isinstance(p, Problem):
            p = getattr(track_generator, "problem", None)
            if not isinstance(p, Problem):
                raise RuntimeError("setTrackGenerator needs a packed Problem")
        p = p.contiguous()
        try:
            p.validate(deep=False)   # sizes; the C ABI checks every element
        except ValueError as e:
            raise _native.MOCError(-1, str(e)) from None
        self.close()
        dims = _native.Dims(p.num_groups, p.num_polar_half, p.num_angles,
                            p.num_materials, p.num_fsrs, p.num_tracks,
                            p.num_segments, p.solve_3d, self._device)
        ctx = C.c_void_p()
        _native.check(self._lib.moc_create(C.byref(dims), C.byref(ctx)))
        self._ctx = ctx
        self._problem = p
        self._call("moc_upload_tracks", _ptr(p.seg_len), _ptr(p.seg_fsr),
                   _ptr(p.seg_off), _ptr(p.track_ang), _ptr(p.next),
                   _ptr(p.flags))
        self._call("moc_upload_quadrature", _ptr(p.weights), _ptr(p.inv_sin))
        self._call("moc_upload_materials", _ptr(p.sigma_t), _ptr(p.sigma_s),
                   _ptr(p.nu_sigma_f), _ptr(p.chi))
        self._call("moc_upload_fsrs", _ptr(p.fsr_mat), _ptr(p.fsr_vol))
        self._call("moc_set_convergence_threshold", self._threshold)
        if self._exp_kind is not None:
            self._call("moc_set_exponential", self._exp_kind)
        if self._shape is not None:
            self._call("moc_set_sweep_shape", *self._shape)
        if self._source_kind != "auto":
            self._call("moc_set_source_kernel", self._SOURCE_KINDS[self._source_kind])
        if self._negative_ok:
            self._call("moc_set_negative_fluxes_allowed", 1)
        if self._keff_balance:
            self._call("moc_set_keff_from_neutron_balance", 1)
        if self._stabilization is not None:
            self._call("moc_set_transport_stabilization", 1, *self._stabilization)
        if self._instances:
            self._call("moc_set_instances", self._instances)
        if self._formation == "otf":
            self._set_otf()
        if self._cmfd is not None:
            self._set_cmfd()
        self._fixed = {}
        self._fixed_by_material = {}
        if p.fixed_sources is not None:
            self._upload_fixed(np.asarray(p.fixed_sources, np.float32))

    def getTrackGenerator(self) -> Optional[Problem]:
        return self._problem

    def setConvergenceThreshold(self, threshold: float) -> None:
        """Solver::setConvergenceThreshold (src/Solver.cpp:461)."""
        if threshold <= 0:
            raise _native.MOCError(-1, "Unable to set the convergence threshold "
                                       f"to {threshold} since it is not positive")
        self._threshold = float(threshold)
        if self._ctx is not None:
            self._call("moc_set_convergence_threshold", self._threshold)

    def getConvergenceThreshold(self) -> float:
        return self._threshold

    def setSegmentFormation(self, formation: str) -> None:
        """"explicit" (stored 3D segments) or "otf": 3D tracks of an extruded
        lattice cut from their radial segments during the sweep
        (TrackGenerator3D::setSegmentFormation(OTF_TRACKS),
        src/TrackGenerator3D.h).  "otf" needs the problem's ``otf`` arrays."""
        if formation not in ("explicit", "otf"):
            raise _native.MOCError(-1, f"unknown segment formation {formation!r}")
        self._formation = formation
        if self._ctx is not None:
            if formation == "otf":
                self._set_otf()
            else:
                self._call("moc_set_otf_tracks", None)

    def getSegmentFormation(self) -> str:
        return self._formation

    def _set_otf(self) -> None:
        o = self._problem.otf
        if o is None:
            raise _native.MOCError(-1, "the problem has no on-the-fly track description")
        arrs = {k: np.ascontiguousarray(v) for k, v in o.items()}
        self._otf_arrays = arrs
        d = _native.OtfTracks(arrs["rad_total"].size, arrs["rad_len"].size,
                              *(_ptr(arrs[k]) for k in ("trk", "trk_f", "ang", "rad_len",
                                                        "rad_fsr", "rad_off", "rad_start",
                                                        "rad_total")),
                              int(arrs["above_fsr"][0]))
        self._call("moc_set_otf_tracks", C.byref(d))

    # ---------------------------------------------------------------- CMFD
    def setCmfd(self, cmfd) -> None:
        """Attaches CMFD acceleration (an ``openmoc_gb300.Cmfd``; None
        detaches it) to computeEigenvalue, as ``Geometry::setCmfd`` does for
        the reference's solvers (src/Geometry.cpp, src/Solver.cpp:1150-1185)."""
        self._cmfd = cmfd
        if self._ctx is not None:
            if cmfd is None:
                self._call("moc_set_cmfd", None)
                self._cmfd_keep = None
            else:
                self._set_cmfd()

    def getCmfd(self):
        return self._cmfd

    def _set_cmfd(self) -> None:
        mesh, keep = self._cmfd.mesh(self._problem)
        self._call("moc_set_cmfd", C.byref(mesh))
        self._cmfd_keep = keep

    def getCmfdInfo(self) -> dict:
        """The last coarse solve: eigenvalue, power iterations, SOR sweeps
        and the prolongation ratio farthest from 1."""
        self._need_ctx()
        en, k, pi, li, mr, fl = (C.c_int(), C.c_double(), C.c_int(), C.c_int(),
                                 C.c_double(), C.c_int())
        self._call("moc_get_cmfd_info", C.byref(en), C.byref(k), C.byref(pi),
                   C.byref(li), C.byref(mr), C.byref(fl))
        return {"enabled": bool(en.value), "keff": k.value,
                "power_iterations": pi.value, "linear_iterations": li.value,
                "max_ratio": mr.value, "failed": bool(fl.value)}

    def getCmfdFluxes(self):
        """(old, new) coarse fluxes of the last coarse solve, [cells][E],
        each normalised to unit total fission source."""
        self._need_ctx()
        if self._cmfd is None:
            raise _native.MOCError(-3, "CMFD is not attached")
        mesh, _ = self._cmfd.mesh(self._problem)
        n = mesh.num_x * mesh.num_y * mesh.num_cmfd_groups
        old = np.zeros(n, np.float64)
        new = np.zeros(n, np.float64)
        self._call("moc_get_cmfd_fluxes", _ptr(old), _ptr(new), n)
        E = mesh.num_cmfd_groups
        return old.reshape(-1, E), new.reshape(-1, E)

    def allowNegativeFluxes(self, negative_fluxes_on: bool) -> None:
        """Solver::allowNegativeFluxes (src/Solver.cpp:623): negative
        sources and fluxes are kept instead of clamped."""
        self._negative_ok = bool(negative_fluxes_on)
        if self._ctx is not None:
            self._call("moc_set_negative_fluxes_allowed", int(self._negative_ok))

    def setKeffFromNeutronBalance(self) -> None:
        """Solver::setKeffFromNeutronBalance (src/Solver.cpp:2045): keff =
        fission / (absorption + leakage) with the leakage tallied at vacuum
        track ends, instead of the ratio of successive fission sources."""
        self._keff_balance = True
        if self._ctx is not None:
            self._call("moc_set_keff_from_neutron_balance", 1)

    def setInstances(self, num_instances: int) -> None:
        """Solves the problem's groups as ``num_instances`` cross-section
        sets side by side (a problem made by ``problem.instances``): one
        sweep per iteration for all of them, sources, keff and the
        normalisation per instance.  No counterpart in OpenMOC."""
        self._instances = int(num_instances)
        if self._ctx is not None:
            self._call("moc_set_instances", self._instances)

    def getInstanceKeffs(self) -> np.ndarray:
        self._need_ctx()
        k = np.zeros(self._instances, np.float64)
        self._call("moc_get_instance_keffs", _ptr(k), self._instances)
        return k

    def getInstanceFluxes(self) -> np.ndarray:
        """[instances, R, G] scalar fluxes."""
        f = self.getFluxes()
        K = self._instances
        return np.ascontiguousarray(
            f.reshape(f.shape[0], K, -1).transpose(1, 0, 2))

    _STABILIZATION = {"DIAGONAL": 0, "YAMAMOTO": 1, "GLOBAL": 2}

    def stabilizeTransport(self, stabilization_factor: float,
                           stabilization_type="DIAGONAL") -> None:
        """Solver::stabilizeTransport (src/Solver.cpp:676): DIAGONAL,
        YAMAMOTO or GLOBAL (names, or 0, 1, 2 as openmoc.DIAGONAL ...)."""
        t = (self._STABILIZATION.get(stabilization_type, -1)
             if isinstance(stabilization_type, str) else int(stabilization_type))
        if t not in (0, 1, 2):
            raise _native.MOCError(-1, f"unknown stabilization type {stabilization_type!r}")
        self._stabilization = (float(stabilization_factor), t)
        if self._ctx is not None:
            self._call("moc_set_transport_stabilization", 1, *self._stabilization)

    def useExponentialInterpolation(self) -> None:
        """Shared-memory table evaluation of 1 - exp(-x) (the default)."""
        self._exp_kind = EXP_TABLE
        if self._ctx is not None:
            self._call("moc_set_exponential", EXP_TABLE)

    def useExponentialIntrinsic(self) -> None:
        """Hardware ex2 evaluation of 1 - exp(-x)."""
        self._exp_kind = EXP_INTRINSIC
        if self._ctx is not None:
            self._call("moc_set_exponential", EXP_INTRINSIC)

    def setSweepShape(self, lanes_per_track_direction: int,
                      group_pairs_per_lane: int) -> None:
        self._shape = (int(lanes_per_track_direction), int(group_pairs_per_lane))
        if self._ctx is not None:
            self._call("moc_set_sweep_shape", *self._shape)

    def getSweepShape(self):
        self._need_ctx()
        a, b = C.c_int(), C.c_int()
        self._call("moc_get_sweep_shape", C.byref(a), C.byref(b))
        return a.value, b.value

    def getExponential(self) -> int:
        """The evaluator in use (EXP_TABLE or EXP_INTRINSIC): the caller's
        choice, or the autotuner's once a solve has run."""
        self._need_ctx()
        k = C.c_int()
        self._call("moc_get_exponential", C.byref(k))
        return k.value

    def setAutotune(self, on: bool) -> None:
        self._need_ctx()
        self._call("moc_set_autotune", int(bool(on)))

    def autotune(self):
        """Times every sweep-kernel shape (and both exponential evaluators
        unless one was chosen) on this problem and keeps the fastest;
        returns (lanes per track direction, groups per lane, evaluator)."""
        self._need_ctx()
        a, b, e = C.c_int(), C.c_int(), C.c_int()
        self._call("moc_autotune", C.byref(a), C.byref(b), C.byref(e))
        return a.value, b.value, e.value

    def getTuningLog(self):
        """[(lanes, groups per lane, evaluator, sweep ms)] of the last tuning."""
        self._need_ctx()
        n = C.c_int()
        cap = 64
        a = np.zeros(cap, np.int32)
        b = np.zeros(cap, np.int32)
        e = np.zeros(cap, np.int32)
        ms = np.zeros(cap, np.float32)
        self._call("moc_get_tuning_log", _ptr(a), _ptr(b), _ptr(e), _ptr(ms), cap,
                   C.byref(n))
        return [(int(a[i]), int(b[i]), int(e[i]), float(ms[i]))
                for i in range(min(n.value, cap))]

    _SOURCE_KINDS = {"auto": 0, "fp32": 1, "tf32x3": 2}

    def setSourceContraction(self, kind: str) -> None:
        """Kernel of computeFSRSources: "fp32" (CUDA cores), "tf32x3" (the
        per-material contraction on the tensor cores with TF32 high/low split
        products, 64 to 96 groups) or "auto" (tf32x3 at >= 70 groups).  No
        counterpart in OpenMOC."""
        if kind not in self._SOURCE_KINDS:
            raise _native.MOCError(-1, f"unknown source contraction {kind!r}")
        self._source_kind = kind
        if self._ctx is not None:
            self._call("moc_set_source_kernel", self._SOURCE_KINDS[kind])

    def getSourceContraction(self) -> str:
        """The source kernel in use: "fp32" or "tf32x3"."""
        self._need_ctx()
        k = C.c_int()
        self._call("moc_get_source_kernel", C.byref(k))
        return {1: "fp32", 2: "tf32x3"}[k.value]

    def setTensorWaitLimit(self, polls: int) -> None:
        """mbarrier polls before the tensor-core source kernel gives up
        waiting (the solve then raises the timeout status); a negative value
        restores the default.  No counterpart in OpenMOC."""
        self._need_ctx()
        self._call("moc_set_tensor_wait_limit", int(polls))

    def setIterationsPerSync(self, k: int) -> None:
        self._need_ctx()
        self._call("moc_set_iterations_per_sync", int(k))

    # ------------------------------------------------------- fixed sources
    def setFixedSourceByFSR(self, fsr_id: int, group: int, source: float) -> None:
        """Solver::setFixedSourceByFSR (src/Solver.cpp:479); group is
        1-based."""
        p = self._problem
        if p is None:
            raise RuntimeError("set a TrackGenerator before fixed sources")
        if group <= 0 or group > p.num_groups:
            raise _native.MOCError(-1, f"Unable to use fixed source for group {group} "
                                       f"in a {p.num_groups} energy group problem")
        if fsr_id < 0 or fsr_id >= p.num_fsrs:
            raise _native.MOCError(-1, f"Unable to use fixed source for FSR {fsr_id} "
                                       f"with only {p.num_fsrs} FSRs in the geometry")
        self._fixed[(int(fsr_id), int(group))] = float(source)
        self._push_fixed()

    def setFixedSourceByMaterial(self, material: int, group: int, source: float) -> None:
        """Solver::setFixedSourceByMaterial: every FSR of the material
        (material given by its index in the packed problem)."""
        p = self._problem
        if p is None:
            raise RuntimeError("set a TrackGenerator before fixed sources")
        if material < 0 or material >= p.num_materials:
            raise _native.MOCError(-1, f"no material {material}")
        if group <= 0 or group > p.num_groups:
            raise _native.MOCError(-1, f"Unable to use fixed source for group {group} "
                                       f"in a {p.num_groups} energy group problem")
        self._fixed_by_material[(int(material), int(group))] = float(source)
        self._push_fixed()

    def setFixedSources(self, sources) -> None:
        """Every FSR's fixed source at once ([R][G]): the bulk form of
        setFixedSourceByFSR over all FSRs and groups."""
        p = self._problem
        if p is None:
            raise RuntimeError("set a TrackGenerator before fixed sources")
        q = np.asarray(sources, np.float32)
        if q.size != p.num_fsrs * p.num_groups:
            raise _native.MOCError(-1, f"fixed sources need {p.num_fsrs} x "
                                       f"{p.num_groups} values, got {q.size}")
        self._fixed = {}
        self._fixed_by_material = {}
        self._upload_fixed(q)

    def resetFixedSources(self) -> None:
        self._fixed = {}
        self._fixed_by_material = {}
        if self._ctx is not None:
            self._call("moc_set_fixed_sources", None)

    def _push_fixed(self) -> None:
        p = self._problem
        q = np.zeros((p.num_fsrs, p.num_groups), np.float32)
        for (m, g), v in self._fixed_by_material.items():
            q[p.fsr_mat == m, g - 1] = v
        for (r, g), v in self._fixed.items():
            q[r, g - 1] = v
        self._upload_fixed(q)

    def _upload_fixed(self, q: np.ndarray) -> None:
        q = np.ascontiguousarray(q, np.float32).ravel()
        self._fixed_array = q
        self._call("moc_set_fixed_sources", _ptr(q))

    # ------------------------------------------------------------- solves
    def computeEigenvalue(self, max_iters: int = 1000,
                          res_type: int = FISSION_SOURCE) -> None:
        """Solver::computeEigenvalue (src/Solver.cpp:1542-1700), run
        device-resident."""
        self._need_ctx()
        t0 = time.perf_counter()
        self._call("moc_compute_eigenvalue", int(max_iters), int(res_type))
        self._total_time = time.perf_counter() - t0
        self._after_solve()

    def computeSource(self, max_iters: int = 1000, k_eff: float = 1.0,
                      res_type: int = TOTAL_SOURCE) -> None:
        """Solver::computeSource (src/Solver.cpp:1459-1535)."""
        self._need_ctx()
        if k_eff <= 0:
            raise _native.MOCError(-1, f"The Solver is unable to compute the source with "
                                       f"keff = {k_eff} since it is not a positive value")
        t0 = time.perf_counter()
        self._call("moc_compute_source", int(max_iters), float(k_eff), int(res_type))
        self._total_time = time.perf_counter() - t0
        self._after_solve()

    def computeFlux(self, max_iters: int = 1000, only_fixed_source: bool = True) -> None:
        """Solver::computeFlux (src/Solver.cpp:1352-1456)."""
        self._need_ctx()
        t0 = time.perf_counter()
        self._call("moc_compute_flux", int(max_iters), int(bool(only_fixed_source)))
        self._total_time = time.perf_counter() - t0
        self._after_solve()

    def _after_solve(self) -> None:
        n = C.c_int()
        self._call("moc_get_num_iterations", C.byref(n))
        self._num_iterations = n.value
        k = C.c_double()
        self._call("moc_get_keff", C.byref(k))
        self._keff = k.value

    # ------------------------------------------------------------ results
    def getKeff(self) -> float:
        if self._ctx is not None:
            k = C.c_double()
            self._call("moc_get_keff", C.byref(k))
            self._keff = k.value
        return self._keff

    def getNumIterations(self) -> int:
        return self._num_iterations

    def getTotalTime(self) -> float:
        return self._total_time

    def getResidual(self) -> float:
        self._need_ctx()
        r = C.c_double()
        self._call("moc_get_residual", C.byref(r))
        return r.value

    def getSweepTime(self):
        """(milliseconds of transport sweeps, number of sweeps) of the last
        solve: the Timer split "Transport Sweep"."""
        self._need_ctx()
        ms, n = C.c_double(), C.c_int64()
        self._call("moc_get_sweep_time", C.byref(ms), C.byref(n))
        return ms.value, n.value

    def getLaunchCount(self) -> int:
        self._need_ctx()
        n = C.c_int64()
        self._call("moc_get_launch_count", C.byref(n))
        return n.value

    def benchIterations(self, steps: int, res_type: int = FISSION_SOURCE,
                        flush_l2: bool = True):
        """Times ``steps`` eigenvalue iterations (convergence exit off) with
        CUDA events on the solver's stream; returns (step_ms, sweep_ms)
        arrays."""
        self._need_ctx()
        st = np.zeros(steps, np.float64)
        sw = np.zeros(steps, np.float64)
        self._call("moc_bench_iterations", int(steps), int(res_type), int(bool(flush_l2)),
                   _ptr(st), _ptr(sw))
        return st, sw

    def evaluateAttenuation(self, x, kind: int) -> np.ndarray:
        """1 - exp(-x) on the GPU with the sweep's evaluator ``kind``."""
        self._need_ctx()
        xa = np.ascontiguousarray(x, np.float32).ravel()
        out = np.empty_like(xa)
        self._call("moc_eval_attenuation", int(kind), _ptr(xa), _ptr(out), xa.size)
        return out

    def getFluxes(self) -> np.ndarray:
        """All scalar fluxes as an [R, G] array (Solver::getFluxes)."""
        self._need_ctx()
        p = self._problem
        out = np.empty(p.num_fsrs * p.num_groups, np.float32)
        self._call("moc_get_fluxes", _ptr(out), out.size)
        return out.reshape(p.num_fsrs, p.num_groups)

    def getFlux(self, fsr_id: int, group: int) -> float:
        """Solver::getFlux (src/Solver.cpp:298-321); group is 1-based."""
        self._need_ctx()
        p = self._problem
        if fsr_id >= p.num_fsrs:
            raise _native.MOCError(-1, f"Unable to return a scalar flux for FSR ID = "
                                       f"{fsr_id} since the max FSR ID = {p.num_fsrs - 1}")
        if fsr_id < 0:
            raise _native.MOCError(-1, f"Unable to return a scalar flux for FSR ID = "
                                       f"{fsr_id} since FSRs do not have negative IDs")
        if group - 1 >= p.num_groups:
            raise _native.MOCError(-1, f"Unable to return a scalar flux in group {group} "
                                       f"since there are only {p.num_groups} groups")
        if group <= 0:
            raise _native.MOCError(-1, f"Unable to return a scalar flux in group {group} "
                                       f"since groups must be greater or equal to 1")
        return float(self.getFluxes()[fsr_id, group - 1])

    def setFluxes(self, fluxes) -> None:
        """Solver::setFluxes: [R, G] (or flat) scalar fluxes."""
        self._need_ctx()
        a = np.ascontiguousarray(fluxes, np.float32).ravel()
        self._call("moc_set_fluxes", _ptr(a), a.size)

    def computeFSRFissionRates(self, num_FSRs: int, nu: bool = False) -> np.ndarray:
        """Solver::computeFSRFissionRates (src/Solver.h:539-540)."""
        self._need_ctx()
        p = self._problem
        if num_FSRs != p.num_fsrs:
            raise _native.MOCError(-1, f"{num_FSRs} FSRs requested, the problem has "
                                       f"{p.num_fsrs}")
        out = np.empty(p.num_fsrs, np.float64)
        self._call("moc_compute_fsr_fission_rates", _ptr(out), out.size, int(bool(nu)))
        return out

    # ------------------------------------------------- per-hook interface
    # The protected hooks of src/Solver.h:334-431, exposed one call each so
    # that a caller can drive (or test) one step of source iteration.
    def zeroTrackFluxes(self):
        self._call("moc_zero_track_fluxes")

    def flattenFSRFluxes(self, value: float):
        self._call("moc_flatten_fsr_fluxes", float(value))

    def flattenFSRFluxesChiSpectrum(self, material: int):
        self._call("moc_flatten_fsr_fluxes_chi", int(material))

    def storeFSRFluxes(self):
        self._call("moc_store_fsr_fluxes")

    def normalizeFluxes(self) -> float:
        f = C.c_double()
        self._call("moc_normalize_fluxes", C.byref(f))
        return f.value

    def computeStabilizingFlux(self):
        self._call("moc_compute_stabilizing_flux")

    def stabilizeFlux(self):
        self._call("moc_stabilize_flux")

    def computeFSRFissionSources(self):
        self._call("moc_compute_fsr_fission_sources")

    def computeFSRScatterSources(self):
        self._call("moc_compute_fsr_scatter_sources")

    def computeFSRSources(self, iteration: int):
        self._call("moc_compute_fsr_sources", int(iteration))

    def transportSweep(self):
        self._call("moc_transport_sweep")

    def addSourceToScalarFlux(self):
        self._call("moc_add_source_to_scalar_flux")

    def computeKeff(self):
        self._call("moc_compute_keff")

    def computeResidual(self, res_type: int) -> float:
        r = C.c_double()
        self._call("moc_compute_residual", int(res_type), C.byref(r))
        return r.value

    def setKeff(self, keff: float):
        self._call("moc_set_keff", float(keff))

    def getReducedSources(self) -> np.ndarray:
        p = self._problem
        out = np.empty(p.num_fsrs * p.num_groups, np.float32)
        self._call("moc_get_reduced_sources", _ptr(out), out.size)
        return out.reshape(p.num_fsrs, p.num_groups)

    def getOldFluxes(self) -> np.ndarray:
        p = self._problem
        out = np.empty(p.num_fsrs * p.num_groups, np.float32)
        self._call("moc_get_old_fluxes", _ptr(out), out.size)
        return out.reshape(p.num_fsrs, p.num_groups)

    def setOldFluxes(self, fluxes) -> None:
        a = np.ascontiguousarray(fluxes, np.float32).ravel()
        self._call("moc_set_old_fluxes", _ptr(a), a.size)

    def getStartFlux(self) -> np.ndarray:
        p = self._problem
        out = np.empty(2 * p.num_tracks * p.fluxes_per_track, np.float32)
        self._call("moc_get_start_flux", _ptr(out), out.size)
        return out

    def setStartFlux(self, psi) -> None:
        a = np.ascontiguousarray(psi, np.float32).ravel()
        self._call("moc_set_start_flux", _ptr(a), a.size)


class GB300LSSolver(GB300Solver):
    """The linear-source solver with OpenMOC's CPULSSolver API
    (``src/CPULSSolver.h``): flat plus linear (x, y) source and flux moments
    per FSR, for 2D tracks.

    The linear-source geometry -- each segment's start relative to its FSR
    centroid, the track direction, azimuthal and polar weights of every angle
    row -- comes from ``linear_source`` or from the problem's own
    ``linear_source`` (``pack_linear_source`` in
    ``openmoc_gb300/adapter/pack_reference.h``, or
    :func:`openmoc_gb300.lattice.lattice`); the expansion matrices and source
    constants are computed on the GPU when the tracks are set.
    """

    def __init__(self, track_generator: Optional[Problem] = None,
                 linear_source: Optional[dict] = None, device: int = 0):
        self._ls = linear_source
        self._fixed_moments = {}
        super().__init__(track_generator, device)

    def setTrackGenerator(self, track_generator: Problem) -> None:
        super().setTrackGenerator(track_generator)
        ls = self._ls if self._ls is not None else self._problem.linear_source
        if ls is None:
            raise _native.MOCError(-1, "the linear-source solver needs segment "
                                       "start positions and angle data")
        self.setLinearSource(ls)

    def setLinearSource(self, ls: dict) -> None:
        """Uploads the linear-source geometry (the keys of
        ``openmoc_gb300.problem.LS_KEYS``) and computes the expansion
        constants."""
        self._need_ctx()
        p = self._problem
        arrs = {}
        keys = [("seg_x", np.float32, p.num_segments),
                ("seg_y", np.float32, p.num_segments),
                ("ang_dir", np.float64, 2 * p.num_angles),
                ("ang_wgt", np.float64, p.num_angles),
                ("pol_sin", np.float64, p.num_angles * p.num_polar_half),
                ("pol_wgt", np.float64, p.num_angles * p.num_polar_half)]
        if p.solve_3d:   # explicit 3D tracks: z starts and cos theta per row
            keys += [("seg_z", np.float32, p.num_segments),
                     ("pol_cos", np.float64, p.num_angles)]
        for k, dt, n in keys:
            if k not in ls:
                raise _native.MOCError(-1, f"linear-source geometry lacks {k}")
            a = np.ascontiguousarray(ls[k], dt).ravel()
            if a.size != n:
                raise _native.MOCError(-1, f"{k} has {a.size} values, expected {n}")
            arrs[k] = a
        self._ls_arrays = arrs
        g = _native.LSGeometry(*(_ptr(arrs[k]) if k in arrs else None for k in (
            "seg_x", "seg_y", "ang_dir", "ang_wgt", "pol_sin", "pol_wgt",
            "seg_z", "pol_cos")))
        self._call("moc_set_linear_source", C.byref(g))
        self._fixed_moments = {}

    def getNumFlatSourceRegions(self) -> int:
        """FSRs whose expansion matrix is singular (flat source there)."""
        self._need_ctx()
        on, n = C.c_int(), C.c_int64()
        self._call("moc_get_linear_source", C.byref(on), C.byref(n))
        return n.value

    # ------------------------------------------------- fixed source moments
    def setFixedSourceMomentByFSR(self, fsr_id: int, group: int, src_x: float,
                                  src_y: float, src_z: float = 0.0) -> None:
        """CPULSSolver::setFixedSourceMomentByFSR (src/CPULSSolver.cpp:
        280-307); group is 1-based, z ignored for 2D tracks."""
        p = self._problem
        if group <= 0 or group > p.num_groups:
            raise _native.MOCError(-1, f"Unable to set fixed source for group {group} "
                                       f"in a {p.num_groups} energy group problem")
        if fsr_id < 0 or fsr_id >= p.num_fsrs:
            raise _native.MOCError(-1, f"Unable to set fixed source for FSR {fsr_id} "
                                       f"with only {p.num_fsrs} FSRs in the geometry")
        self._fixed_moments[(int(fsr_id), int(group))] = (float(src_x), float(src_y),
                                                          float(src_z))
        m = np.zeros((p.num_fsrs, 3, p.num_groups), np.float32)
        for (r, g), v in self._fixed_moments.items():
            m[r, :, g - 1] = v
        self.setFixedSourceMoments(m)

    def setFixedSourceMoments(self, moments) -> None:
        """Every FSR's fixed source moments at once, [R, 3, G] (x, y, z)."""
        self._need_ctx()
        a = np.ascontiguousarray(moments, np.float32).ravel()
        self._fixed_moment_array = a
        self._call("moc_set_fixed_source_moments", _ptr(a), a.size)

    def resetFixedSources(self) -> None:
        super().resetFixedSources()
        self._fixed_moments = {}
        if self._ctx is not None:
            self._call("moc_set_fixed_source_moments", None, 0)

    # ------------------------------------------------------------- results
    def _moments(self, fn: str) -> np.ndarray:
        self._need_ctx()
        p = self._problem
        out = np.empty(p.num_fsrs * 3 * p.num_groups, np.float32)
        self._call(fn, _ptr(out), out.size)
        return out.reshape(p.num_fsrs, 3, p.num_groups)

    def getFluxMoments(self) -> np.ndarray:
        """The flux moments [R, 3, G] (x, y, z), CPULSSolver::_scalar_flux_xyz."""
        return self._moments("moc_get_flux_moments")

    def setFluxMoments(self, moments) -> None:
        self._need_ctx()
        a = np.ascontiguousarray(moments, np.float32).ravel()
        self._call("moc_set_flux_moments", _ptr(a), a.size)

    def getSourceMoments(self) -> np.ndarray:
        """The reduced source moments [R, 3, G], _reduced_sources_xyz."""
        return self._moments("moc_get_source_moments")

    def getLinearExpansion(self):
        """(inverse expansion matrices [R, NC], source constants [R, NC, G]):
        getLinearExpansionCoeffsBuffer / getSourceConstantsBuffer; NC = 3
        (xx, yy, xy) in 2D, 6 (xx, yy, xy, xz, yz, zz) on 3D tracks."""
        self._need_ctx()
        p = self._problem
        nc = 6 if p.solve_3d else 3
        il = np.empty(nc * p.num_fsrs, np.float64)
        sc = np.empty(nc * p.num_fsrs * p.num_groups, np.float32)
        self._call("moc_get_linear_expansion", _ptr(il), _ptr(sc))
        return il.reshape(p.num_fsrs, nc), sc.reshape(p.num_fsrs, nc, p.num_groups)

    def getFluxByPosition(self, fsr_id: int, dx: float, dy: float,
                          group: int, dz: float = 0.0) -> float:
        """The linear flux at offset (dx, dy[, dz]) from the FSR's centroid:
        CPULSSolver::getFluxByCoords (src/CPULSSolver.cpp:1082-1133) with the
        point given relative to the centroid."""
        il, _ = self.getLinearExpansion()
        m = self.getFluxMoments()[fsr_id, :, group - 1]
        flat = float(self.getFluxes()[fsr_id, group - 1])
        if il.shape[1] == 3:
            a, b, c = il[fsr_id]
            return flat + dx * (a * m[0] + c * m[1]) + dy * (c * m[0] + b * m[1])
        xx, yy, xy, xz, yz, zz = il[fsr_id]
        return (flat + dx * (xx * m[0] + xy * m[1] + xz * m[2])
                + dy * (xy * m[0] + yy * m[1] + yz * m[2])
                + dz * (xz * m[0] + yz * m[1] + zz * m[2]))
