"""CMFD acceleration settings: the Python face of ``moc_cmfd_mesh``.

Mirrors the reference's ``openmoc.Cmfd`` (src/Cmfd.h) for what its
eigenvalue acceleration of 2D problems (flat or linear source) uses: lattice structure
and widths, group structure, CMFD and SOR relaxation factors, flux
limiting, unbounded iterations.  Attach it with ``GB300Solver.setCmfd``
(the reference attaches it to the Geometry, ``Geometry::setCmfd``).

The mesh is laid over the problem's ``cmfd_geometry``: each FSR goes to the
coarse cell holding its lattice cell (an FSR cut by a mesh line raises, as
the reference would have split it), each track end on the boundary to the
face it leaves through.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

from . import _native

VACUUM = 0
REFLECTIVE = 1


class Cmfd:
    """Settings of the coarse-mesh finite-difference accelerator."""

    def __init__(self):
        self._nx = 0
        self._ny = 0
        self._widths: Optional[List[np.ndarray]] = None
        self._groups: Optional[List[List[int]]] = None
        self._relaxation = 0.7          # src/Cmfd.cpp:71
        self._sor = 1.5                 # src/Cmfd.cpp:42
        self._flux_limiting = True      # src/Cmfd.cpp:39
        self._unbounded = 0             # src/Cmfd.cpp:35
        self._edc = True
        self._host = False
        self._device_solve = 0
        self._k_nearest = 0
        self._fsr_cell: Optional[np.ndarray] = None

    # ------------------------------------------------------------ settings
    def setLatticeStructure(self, num_x: int, num_y: int, num_z: int = 1) -> None:
        """Cmfd::setLatticeStructure (src/Cmfd.cpp:2028); 2D only."""
        if num_z != 1:
            raise _native.MOCError(_native.MOC_ERR_UNSUPPORTED,
                                   "CMFD is supported on 2D meshes")
        if num_x < 1 or num_y < 1:
            raise _native.MOCError(-1, "CMFD lattice dimensions must be positive")
        self._nx, self._ny = int(num_x), int(num_y)

    def getNumX(self) -> int:
        return self._nx

    def getNumY(self) -> int:
        return self._ny

    def setWidths(self, widths: Sequence[Sequence[float]]) -> None:
        """Cmfd::setWidths (src/Cmfd.cpp:5569): [widths_x, widths_y]; sets
        the lattice structure from their lengths."""
        wx = np.asarray(widths[0], np.float64)
        wy = np.asarray(widths[1], np.float64)
        if len(widths) > 2 and len(widths[2]) > 1:
            raise _native.MOCError(_native.MOC_ERR_UNSUPPORTED,
                                   "CMFD is supported on 2D meshes")
        if (wx <= 0).any() or (wy <= 0).any():
            raise _native.MOCError(-1, "CMFD cell widths must be positive")
        self._widths = [wx, wy]
        self._nx, self._ny = wx.size, wy.size

    def setGroupStructure(self, group_indices: Sequence[Sequence[int]]) -> None:
        """Cmfd::setGroupStructure (src/Cmfd.cpp:1768): lists of 1-based
        groups, contiguous and in order, e.g. [[1, 2, 3], [4, 5, 6, 7]]."""
        groups = [list(map(int, g)) for g in group_indices]
        flat = [g for grp in groups for g in grp]
        if not groups or any(not g for g in groups) or flat != list(range(1, len(flat) + 1)):
            raise _native.MOCError(-1, "CMFD groups must be contiguous, in "
                                       "order and start at group 1")
        self._groups = groups

    def getNumCmfdGroups(self) -> int:
        return len(self._groups) if self._groups else 0

    def setCMFDRelaxationFactor(self, factor: float) -> None:
        """Cmfd::setCMFDRelaxationFactor (src/Cmfd.cpp:1717)."""
        if not 0.0 < factor <= 1.0:
            raise _native.MOCError(-1, "the CMFD relaxation factor must be in (0, 1]")
        self._relaxation = float(factor)

    def setSORRelaxationFactor(self, factor: float) -> None:
        """Cmfd::setSORRelaxationFactor (src/Cmfd.cpp:1703)."""
        if not 0.0 < factor < 2.0:
            raise _native.MOCError(-1, "The successive over-relaxation factor "
                                       f"must be > 0 and < 2. Input value: {factor}")
        self._sor = float(factor)

    def useFluxLimiting(self, on: bool) -> None:
        """Cmfd::useFluxLimiting (src/Cmfd.cpp:2745)."""
        self._flux_limiting = bool(on)

    def setNumUnboundedIterations(self, n: int) -> None:
        """Cmfd::setNumUnboundedIterations (src/Cmfd.cpp:3407)."""
        self._unbounded = int(n)

    def useLarsenEDC(self, on: bool) -> None:
        """Larsen's effective diffusion coefficient correction (on in the
        reference's flat-source CMFD; never applied with a linear source)."""
        self._edc = bool(on)

    def useHostSolver(self, on: bool) -> None:
        """Solve the coarse problem on the host in FP64 (the tallies go to
        the host and the ratios back every iteration) instead of on the GPU
        in FP32 (the default: one block, no host round trip)."""
        self._host = bool(on)

    def setDeviceSolver(self, kind: str) -> None:
        """Which device kernel runs the coarse power iteration: "auto" (the
        cell-parallel solve, one thread per coarse cell over a cluster of
        blocks, for up to 8 coarse groups and meshes it can map; else one
        block), "block" (one block, any mesh) or "cells" (the cell-parallel
        solve, an error where it does not apply)."""
        kinds = {"auto": 0, "block": 2, "cells": 3}
        if kind not in kinds:
            raise _native.MOCError(-1, f"unknown CMFD device solver {kind!r}")
        self._device_solve = kinds[kind]

    def setKNearest(self, k: int) -> None:
        """Cmfd::setKNearest (src/Cmfd.cpp:3417): each FSR's update ratio
        weighted over the k nearest of the 3 x 3 cells around it by the
        distance from its centroid (k in 1..9)."""
        if not 1 <= int(k) <= 9:
            raise _native.MOCError(-1, "Unable to set CMFD k-nearest to "
                                       f"{k}. k-nearest must be between 1 and 9.")
        self._k_nearest = int(k)

    def setFSRCells(self, fsr_cell: np.ndarray) -> None:
        """The coarse cell of every FSR given directly (iy * num_x + ix, iy
        from y-min), instead of from the problem's lattice-cell boxes."""
        self._fsr_cell = np.ascontiguousarray(fsr_cell, np.int32)

    # ------------------------------------------------------------- binding
    def mesh(self, problem) -> "tuple[_native.CmfdMesh, list]":
        """The moc_cmfd_mesh for `problem` and the arrays it points into
        (kept alive by the caller)."""
        geo = problem.cmfd_geometry
        if geo is None:
            raise _native.MOCError(-1, "the problem has no CMFD geometry (2D "
                                       "lattice problems carry one)")
        bounds = np.asarray(geo["bounds"], np.float64)
        if self._widths is None:
            if "widths_x" in geo and self._nx in (0, geo["widths_x"].size) \
                    and self._ny in (0, geo["widths_y"].size):
                wx = np.asarray(geo["widths_x"], np.float64)
                wy = np.asarray(geo["widths_y"], np.float64)
            else:
                if self._nx < 1 or self._ny < 1:
                    raise _native.MOCError(-1, "set the CMFD lattice structure first")
                wx = np.full(self._nx, (bounds[1] - bounds[0]) / self._nx)
                wy = np.full(self._ny, (bounds[3] - bounds[2]) / self._ny)
        else:
            wx, wy = self._widths
        nx, ny = wx.size, wy.size
        if self._fsr_cell is not None:
            cell = self._fsr_cell
        elif "fsr_box" in geo:
            cell = _cells_of_boxes(np.asarray(geo["fsr_box"], np.float64), bounds, wx, wy)
        elif "fsr_cell" in geo and geo["widths_x"].size == nx and geo["widths_y"].size == ny:
            cell = np.ascontiguousarray(geo["fsr_cell"], np.int32)
        else:
            raise _native.MOCError(-1, "no FSR-to-cell map for this CMFD mesh")
        G = problem.num_groups
        if self._groups is None:
            group_of = np.arange(G, dtype=np.int32)
            E = G
        else:
            if sum(len(g) for g in self._groups) != G:
                raise _native.MOCError(-1, "the CMFD group structure does not "
                                           f"cover the {G} energy groups")
            group_of = np.concatenate([np.full(len(g), e, np.int32)
                                       for e, g in enumerate(self._groups)])
            E = len(self._groups)
        end = np.ascontiguousarray(geo["end_face"], np.int8)
        if self._edc:
            mu = np.ascontiguousarray(geo["edc_mu"], np.float64)
            w = np.ascontiguousarray(geo["edc_w"], np.float64)
        else:
            mu = w = np.zeros(0, np.float64)
        wx = np.ascontiguousarray(wx, np.float64)
        wy = np.ascontiguousarray(wy, np.float64)
        bc = np.asarray(geo["bc"], np.int32)
        cen = np.zeros(0, np.float64)
        if self._k_nearest > 0:
            if "fsr_centroid" in geo:
                cen = np.ascontiguousarray(geo["fsr_centroid"], np.float64)
            elif problem.linear_source is not None and "centroid" in problem.linear_source:
                cen = np.ascontiguousarray(problem.linear_source["centroid"], np.float64)
            else:
                raise _native.MOCError(-1, "the k-nearest update needs the FSR "
                                           "centroids")
        keep = [wx, wy, cell, end, group_of, mu, w, cen]
        ptr = lambda a: a.ctypes.data if a.size else None  # noqa: E731
        m = _native.CmfdMesh(nx, ny, ptr(wx), ptr(wy), ptr(cell), ptr(end),
                             (_native.C.c_int32 * 4)(*[int(b) for b in bc]),
                             E, ptr(group_of), int(mu.size), ptr(mu), ptr(w),
                             self._relaxation, self._sor,
                             1 if self._flux_limiting else 0, self._unbounded,
                             1 if self._host else self._device_solve, self._k_nearest, ptr(cen),
                             float(bounds[0]), float(bounds[2]))
        return m, keep


def _cells_of_boxes(box: np.ndarray, bounds: np.ndarray, wx: np.ndarray,
                    wy: np.ndarray) -> np.ndarray:
    """Coarse cell of every FSR from the box of its lattice cell; a box
    that a mesh line crosses raises."""
    ex = bounds[0] + np.concatenate([[0.0], np.cumsum(wx)])
    ey = bounds[2] + np.concatenate([[0.0], np.cumsum(wy)])
    if abs(ex[-1] - bounds[1]) > 1e-6 * max(1.0, abs(bounds[1])) or \
            abs(ey[-1] - bounds[3]) > 1e-6 * max(1.0, abs(bounds[3])):
        raise _native.MOCError(-1, "the CMFD widths do not span the geometry")
    tol = 1e-9 * max(1.0, float(np.abs(bounds).max()))
    cx = (box[:, 0] + box[:, 1]) * 0.5
    cy = (box[:, 2] + box[:, 3]) * 0.5
    ix = np.clip(np.searchsorted(ex, cx, side="right") - 1, 0, wx.size - 1)
    iy = np.clip(np.searchsorted(ey, cy, side="right") - 1, 0, wy.size - 1)
    if ((box[:, 0] < ex[ix] - tol) | (box[:, 1] > ex[ix + 1] + tol) |
            (box[:, 2] < ey[iy] - tol) | (box[:, 3] > ey[iy + 1] + tol)).any():
        raise _native.MOCError(-1, "a CMFD mesh line cuts a lattice cell: the "
                                   "mesh must follow the lattice")
    return np.ascontiguousarray(iy * wx.size + ix, np.int32)
