"""Batched solve server: many independent eigenvalue and fixed-source solves
of uneven size sharing one GPU (ctypes binding of
``include/openmoc_gb300_serve.h``).

OpenMOC runs one problem per ``Solver`` object, one at a time
(src/Solver.cpp:1352-1700).  A :class:`Server` runs the same loop body for
every admitted request at once: one pool per (groups, polar) count and
source kind (flat, or linear as CPULSSolver) holds its solves in shared
device arrays, an iteration is six kernel launches for
all of them, blocks of iterations replay as CUDA graphs, and finished solves
are retired and queued ones admitted between blocks (continuous batching).

Example::

    srv = Server(iterations_per_poll=8)
    srv.add_pool(num_groups=7, num_polar_half=3, max_solves=64, ...)
    t = srv.submit(problem, kind="eigenvalue", threshold=1e-5)
    srv.start()
    res = srv.wait(t)          # dict: keff, iterations, flux [R][G], times
    srv.close()
"""
from __future__ import annotations

import ctypes as C
import threading
from typing import Dict, List, Optional

import numpy as np

from . import _native
from .problem import Problem

SOLVE_EIGENVALUE = 0
SOLVE_SOURCE = 1
SOLVE_FLUX = 2
_KINDS = {"eigenvalue": SOLVE_EIGENVALUE, "source": SOLVE_SOURCE, "flux": SOLVE_FLUX}


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("iterations_per_poll", C.c_int32),
                ("use_graphs", C.c_int32), ("priorities", C.c_int32),
                ("hot_bytes", C.c_int64)]


class PoolConfig(C.Structure):
    _fields_ = [
        ("num_groups", C.c_int32), ("num_polar_half", C.c_int32),
        ("max_solves", C.c_int32), ("max_materials", C.c_int32),
        ("max_angles", C.c_int32), ("max_fsrs", C.c_int64),
        ("max_tracks", C.c_int64), ("max_segments", C.c_int64),
        ("lanes", C.c_int32), ("pairs", C.c_int32), ("exp_kind", C.c_int32),
        ("linear_source", C.c_int32),
    ]


class Request(C.Structure):
    _fields_ = [
        ("num_groups", C.c_int32), ("num_polar_half", C.c_int32),
        ("num_angles", C.c_int32), ("num_materials", C.c_int32),
        ("num_fsrs", C.c_int64), ("num_tracks", C.c_int64),
        ("num_segments", C.c_int64),
        ("seg_len", C.c_void_p), ("seg_fsr", C.c_void_p), ("seg_off", C.c_void_p),
        ("track_ang", C.c_void_p), ("next", C.c_void_p), ("flags", C.c_void_p),
        ("weights", C.c_void_p), ("inv_sin", C.c_void_p),
        ("sigma_t", C.c_void_p), ("sigma_s", C.c_void_p),
        ("nu_sigma_f", C.c_void_p), ("chi", C.c_void_p),
        ("fsr_mat", C.c_void_p), ("fsr_vol", C.c_void_p),
        ("fixed_source", C.c_void_p),
        ("kind", C.c_int32), ("max_iters", C.c_int32), ("res_type", C.c_int32),
        ("k_eff", C.c_double), ("threshold", C.c_double),
        ("flux_out", C.c_void_p), ("allow_negative_fluxes", C.c_int32),
        ("linear_source", C.POINTER(_native.LSGeometry)),
        ("fixed_source_moments", C.c_void_p), ("moments_out", C.c_void_p),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("iterations", C.c_int32), ("converged", C.c_int32),
        ("pool", C.c_int32), ("keff", C.c_double), ("residual", C.c_double),
        ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "submitted", "admitted", "completed", "failed", "blocks",
        "graph_captures", "kernel_launches", "live", "queued")] + [
        (n, C.c_double) for n in (
            "gpu_busy_s", "host_admit_s", "host_retire_s", "host_graph_s")]


class PoolStats(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "num_groups", "num_polar_half", "lanes", "pairs", "exp_kind", "live")] + [
        (n, C.c_int64) for n in ("admitted", "completed", "blocks", "tunes")] + [
        ("gpu_busy_s", C.c_double)]


_P = C.c_void_p
_SIGS = {
    "moc_server_create": ([C.POINTER(ServerConfig), C.POINTER(C.c_void_p)], C.c_int),
    "moc_server_destroy": ([_P], C.c_int),
    "moc_server_add_pool": ([_P, C.POINTER(PoolConfig), C.POINTER(C.c_int)], C.c_int),
    "moc_server_submit": ([_P, C.POINTER(Request), C.POINTER(C.c_int64)], C.c_int),
    "moc_server_step": ([_P, C.POINTER(C.c_int64)], C.c_int),
    "moc_server_start": ([_P], C.c_int),
    "moc_server_stop": ([_P], C.c_int),
    "moc_server_wait": ([_P, C.c_int64, C.c_double, C.POINTER(Result)], C.c_int),
    "moc_server_poll": ([_P, _P, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "moc_server_stats_get": ([_P, C.POINTER(Stats)], C.c_int),
    "moc_server_loop_error": ([_P], C.c_char_p),
    "moc_server_pool_stats": ([_P, C.c_int, C.POINTER(PoolStats)], C.c_int),
}

_bound = False
_bind_lock = threading.Lock()


def _lib():
    global _bound
    L = _native.lib()
    with _bind_lock:
        if not _bound:
            for name, (args, res) in _SIGS.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            _bound = True
    return L


def exported_symbols() -> List[str]:
    return list(_SIGS)


def pool_capacity(problems, max_solves: int) -> Dict[str, int]:
    """Capacity that holds max_solves copies of the largest of `problems`
    in every dimension at once (no fragmentation stalls)."""
    def most(f):
        return max(f(p) for p in problems)
    return dict(
        max_solves=max_solves,
        max_materials=min(256, max_solves * most(lambda p: p.num_materials)),
        max_angles=max_solves * most(lambda p: p.num_angles),
        max_fsrs=max_solves * most(lambda p: p.num_fsrs),
        max_tracks=max_solves * most(lambda p: p.num_tracks + 1),
        max_segments=max_solves * most(lambda p: max(p.num_segments, 1)),
    )


class Server:
    """The request loop.  Requests are validated and packed on submit; the
    arrays they reference are kept alive here until they complete."""

    def __init__(self, device: int = 0, iterations_per_poll: int = 8,
                 use_graphs: bool = True, priorities: bool = True,
                 hot_bytes: int = 0):
        """hot_bytes caps the sources and tallies (8 B per FSR and group)
        of all live solves, to keep the sweep's gathers in L2 (0: no
        cap)."""
        L = _lib()
        cfg = ServerConfig(device, iterations_per_poll, 1 if use_graphs else 0,
                           1 if priorities else 0, int(hot_bytes))
        h = C.c_void_p()
        _native.check(L.moc_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep: Dict[int, tuple] = {}
        self._running = False

    # ---- set-up ---------------------------------------------------------
    def add_pool(self, num_groups: int, num_polar_half: int, max_solves: int,
                 max_materials: int, max_angles: int, max_fsrs: int,
                 max_tracks: int, max_segments: int,
                 shape: Optional[tuple] = None,
                 linear_source: bool = False) -> int:
        """Adds the pool of (num_groups, num_polar_half) and source kind
        (linear_source: the pool takes linear-source requests, solved as
        CPULSSolver).  shape = (lanes, pairs, exp_kind) fixes the sweep
        shape; None autotunes it on the pool's first batch."""
        lanes, pairs, kind = shape if shape else (0, 0, 0)
        cfg = PoolConfig(num_groups, num_polar_half, max_solves, max_materials,
                         max_angles, max_fsrs, max_tracks, max_segments,
                         lanes, pairs, kind, 1 if linear_source else 0)
        idx = C.c_int()
        _native.check(_lib().moc_server_add_pool(self._h, C.byref(cfg), C.byref(idx)))
        return idx.value

    # ---- requests ---------------------------------------------------------
    def submit(self, p: Problem, kind: str = "eigenvalue", max_iters: int = 1000,
               res_type: int = 1, k_eff: float = 1.0, threshold: float = 1e-5,
               fixed_source: Optional[np.ndarray] = None,
               linear_source=False,
               fixed_source_moments: Optional[np.ndarray] = None,
               allow_negative_fluxes: bool = False) -> int:
        """Queues a solve of `p`; returns its ticket.  kind "eigenvalue" is
        Solver.computeEigenvalue(max_iters, res_type); "source" is
        Solver.computeSource(max_iters, k_eff, res_type) with fixed_source
        (default: p.fixed_sources) as [R][G] source; "flux" is
        Solver.computeFlux(max_iters, True): that fixed source alone,
        SCALAR_FLUX residual.  linear_source (True: p.linear_source, or a
        dict of the same arrays) solves it as CPULSSolver in the linear-
        source pool of its group and polar count, with fixed_source_moments
        [R][3][G] (CPULSSolver.setFixedSourceMomentByFSR); the result then
        carries the flux moments [R][3][G].  allow_negative_fluxes is
        Solver.allowNegativeFluxes(True)."""
        arrs = dict(
            seg_len=np.ascontiguousarray(p.seg_len, np.float32),
            seg_fsr=np.ascontiguousarray(p.seg_fsr, np.int32),
            seg_off=np.ascontiguousarray(p.seg_off, np.int64),
            track_ang=np.ascontiguousarray(p.track_ang, np.int32),
            next=np.ascontiguousarray(p.next, np.int64).ravel(),
            flags=np.ascontiguousarray(p.flags, np.uint8),
            weights=np.ascontiguousarray(p.weights, np.float32),
            inv_sin=np.ascontiguousarray(p.inv_sin, np.float32),
            sigma_t=np.ascontiguousarray(p.sigma_t, np.float32),
            sigma_s=np.ascontiguousarray(p.sigma_s, np.float32),
            nu_sigma_f=np.ascontiguousarray(p.nu_sigma_f, np.float32),
            chi=np.ascontiguousarray(p.chi, np.float32),
            fsr_mat=np.ascontiguousarray(p.fsr_mat, np.int32),
            fsr_vol=np.ascontiguousarray(p.fsr_vol, np.float32),
        )
        fs = fixed_source if fixed_source is not None else p.fixed_sources
        if fs is not None:
            arrs["fixed_source"] = np.ascontiguousarray(fs, np.float32).reshape(
                p.num_fsrs, p.num_groups)
        flux = np.zeros((p.num_fsrs, p.num_groups), np.float32)
        ls = p.linear_source if linear_source is True else (linear_source or None)
        if linear_source is True and ls is None:
            raise _native.MOCError(-1, "the problem has no linear-source geometry")
        moments = geom = None
        if ls is not None:
            for k, dt in (("seg_x", np.float32), ("seg_y", np.float32),
                          ("ang_dir", np.float64), ("ang_wgt", np.float64),
                          ("pol_sin", np.float64), ("pol_wgt", np.float64)):
                if k not in ls:
                    raise _native.MOCError(-1, f"linear-source geometry lacks {k}")
                arrs["ls_" + k] = np.ascontiguousarray(ls[k], dt).ravel()
            for k, n in (("seg_x", p.num_segments), ("seg_y", p.num_segments),
                         ("ang_dir", 2 * p.num_angles), ("ang_wgt", p.num_angles),
                         ("pol_sin", p.num_angles * p.num_polar_half),
                         ("pol_wgt", p.num_angles * p.num_polar_half)):
                if arrs["ls_" + k].size != n:
                    raise _native.MOCError(
                        -1, f"{k} has {arrs['ls_' + k].size} values, expected {n}")
            geom = _native.LSGeometry(*(arrs["ls_" + k].ctypes.data for k in (
                "seg_x", "seg_y", "ang_dir", "ang_wgt", "pol_sin", "pol_wgt")))
            moments = np.zeros((p.num_fsrs, 3, p.num_groups), np.float32)
            if fixed_source_moments is not None:
                arrs["fixed_source_moments"] = np.ascontiguousarray(
                    fixed_source_moments, np.float32).reshape(
                        p.num_fsrs, 3, p.num_groups)
        elif fixed_source_moments is not None:
            raise _native.MOCError(-1, "fixed source moments need a linear source")
        req = Request()
        req.num_groups = p.num_groups
        req.num_polar_half = p.num_polar_half
        req.num_angles = p.num_angles
        req.num_materials = p.num_materials
        req.num_fsrs = p.num_fsrs
        req.num_tracks = p.num_tracks
        req.num_segments = p.num_segments
        for k, a in arrs.items():
            if not k.startswith("ls_"):
                setattr(req, k, a.ctypes.data)
        req.kind = _KINDS[kind]
        req.max_iters = max_iters
        req.res_type = res_type
        req.k_eff = k_eff
        req.threshold = threshold
        req.flux_out = flux.ctypes.data
        req.allow_negative_fluxes = 1 if allow_negative_fluxes else 0
        if geom is not None:
            req.linear_source = C.pointer(geom)
            req.moments_out = moments.ctypes.data
        t = C.c_int64()
        _native.check(_lib().moc_server_submit(self._h, C.byref(req), C.byref(t)))
        self._keep[t.value] = (req, arrs, geom, flux, moments)
        return t.value

    def step(self) -> int:
        """One pass of the loop on this thread; returns live + queued."""
        n = C.c_int64()
        _native.check(_lib().moc_server_step(self._h, C.byref(n)))
        return n.value

    def run_until_idle(self) -> None:
        while self.step() > 0:
            pass

    def start(self) -> None:
        _native.check(_lib().moc_server_start(self._h))
        self._running = True

    def stop(self) -> None:
        _native.check(_lib().moc_server_stop(self._h))
        self._running = False

    def wait(self, ticket: int, timeout: Optional[float] = None) -> dict:
        r = Result()
        _native.check(_lib().moc_server_wait(
            self._h, ticket, -1.0 if timeout is None else float(timeout), C.byref(r)))
        _, _, _, flux, moments = self._keep.pop(ticket)
        if r.status != 0:
            why = self.loop_error()
            raise _native.MOCError(r.status, f"request {ticket} failed"
                                   + (f": {why}" if why else ""))
        out = dict(keff=r.keff, iterations=r.iterations, converged=bool(r.converged),
                   residual=r.residual, pool=r.pool, flux=flux,
                   t_submit=r.t_submit, t_admit=r.t_admit, t_done=r.t_done)
        if moments is not None:
            out["moments"] = moments
        return out

    def poll(self) -> List[int]:
        buf = (C.c_int64 * 1024)()
        n = C.c_int()
        out: List[int] = []
        while True:
            _native.check(_lib().moc_server_poll(self._h, buf, 1024, C.byref(n)))
            out.extend(buf[i] for i in range(n.value))
            if n.value < 1024:
                return out

    def loop_error(self) -> str:
        """The last error inside the request loop ("" when none): the call
        that failed, which failed the requests of its pool."""
        return (_lib().moc_server_loop_error(self._h) or b"").decode()

    def stats(self) -> dict:
        s = Stats()
        _native.check(_lib().moc_server_stats_get(self._h, C.byref(s)))
        return {n: getattr(s, n) for n, _ in Stats._fields_}

    def pool_stats(self, pool: int) -> dict:
        s = PoolStats()
        _native.check(_lib().moc_server_pool_stats(self._h, pool, C.byref(s)))
        return {n: getattr(s, n) for n, _ in PoolStats._fields_}

    def close(self) -> None:
        if self._h:
            _lib().moc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
