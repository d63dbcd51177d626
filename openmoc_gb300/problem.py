"""Packed MOC problems: tracks, segments, quadrature and cross sections.

A :class:`Problem` holds, as flat numpy arrays, everything the transport
sweep reads.  It is what OpenMOC's ``TrackGenerator`` + ``Geometry`` +
``Material`` objects contain once tracks have been generated and segmented
(``src/Track.h:27-58``, ``src/TrackGenerator.cpp:796-880``,
``src/Material.h:81-103``), laid out for one copy each to the GPU:

============  =======  =========  ===========================================
name          dtype    shape      meaning
============  =======  =========  ===========================================
seg_len       float32  [S]        segment length (cm)
seg_fsr       int32    [S]        flat source region of the segment
seg_off       int64    [T+1]      first segment of each track (UID order)
track_ang     int32    [T]        row of ``weights``/``inv_sin`` of the track
next          int64    [2T]       next track forward / backward
flags         uint8    [T]        bit0 next-fwd enters forward, bit1
                                  next-bwd enters forward, bit2/bit3 the
                                  forward/backward flux is transferred
weights       float32  [A, Ph]    total quadrature weight w(a, p)
inv_sin       float32  [A, Ph]    1 / sin(theta_p) (1 for 3D tracks)
sigma_t       float32  [M, G]     total cross section
sigma_s       float32  [M, G, G]  scattering, [dest, orig]
nu_sigma_f    float32  [M, G]
chi           float32  [M, G]
fsr_mat       int32    [R]        material of each FSR
fsr_vol       float32  [R]        FSR volume (area in 2D)
============  =======  =========  ===========================================

The same layout is declared for the C ABI in ``include/openmoc_gb300.h``.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field
from typing import Dict, Optional, Tuple

import numpy as np

_ARRAY_DTYPES = {
    "seg_len": np.float32,
    "seg_fsr": np.int32,
    "seg_off": np.int64,
    "track_ang": np.int32,
    "next": np.int64,
    "flags": np.uint8,
    "weights": np.float32,
    "inv_sin": np.float32,
    "sigma_t": np.float32,
    "sigma_s": np.float32,
    "nu_sigma_f": np.float32,
    "chi": np.float32,
    "fsr_mat": np.int32,
    "fsr_vol": np.float32,
}

LS_KEYS = ("seg_x", "seg_y", "ang_dir", "ang_wgt", "pol_sin", "pol_wgt")
# the explicit 3D tracks' extra linear-source arrays
LS_KEYS_3D = ("seg_z", "pol_cos")
LS_DTYPES = {"seg_x": np.float32, "seg_y": np.float32, "ang_dir": np.float64,
             "ang_wgt": np.float64, "pol_sin": np.float64, "pol_wgt": np.float64,
             "centroid": np.float64, "seg_z": np.float32, "pol_cos": np.float64}

FLAG_NEXT_FWD_IS_FWD = 1
FLAG_NEXT_BWD_IS_FWD = 2
FLAG_TRANSFER_FWD = 4
FLAG_TRANSFER_BWD = 8


@dataclass
class Problem:
    num_groups: int
    num_polar_half: int
    num_angles: int
    num_materials: int
    num_fsrs: int
    num_tracks: int
    num_segments: int
    solve_3d: int
    seg_len: np.ndarray
    seg_fsr: np.ndarray
    seg_off: np.ndarray
    track_ang: np.ndarray
    next: np.ndarray
    flags: np.ndarray
    weights: np.ndarray
    inv_sin: np.ndarray
    sigma_t: np.ndarray
    sigma_s: np.ndarray
    nu_sigma_f: np.ndarray
    chi: np.ndarray
    fsr_mat: np.ndarray
    fsr_vol: np.ndarray
    fixed_sources: Optional[np.ndarray] = None
    meta: Dict[str, float] = field(default_factory=dict)
    # Linear-source geometry (CPULSSolver): seg_x, seg_y [S] float32
    # start of each segment relative to its FSR centroid; ang_dir [A][2]
    # cos/sin phi, ang_wgt [A] azimuthal spacing x weight, pol_sin and
    # pol_wgt [A][Ph] (float64); optionally centroid [R][2] (float64).  For
    # explicit 3D tracks also seg_z [S] and pol_cos [A] (cos theta of each
    # angle row), pol_wgt being polar spacing x polar weight, centroid
    # [R][3].
    linear_source: Optional[Dict[str, np.ndarray]] = None
    # On-the-fly description of extruded 3D tracks (moc_otf_tracks arrays:
    # trk, trk_f, ang, rad_len, rad_fsr, rad_off, rad_start, rad_total,
    # above_fsr); the explicit segments above stay valid.
    otf: Optional[Dict[str, np.ndarray]] = None
    # What a CMFD mesh is laid over (2D): end_face [T][2] int8 boundary face
    # crossed where each track's forward / backward traversal leaves the
    # geometry (0 x-min, 1 y-min, 2 x-max, 3 y-max, -1 none); bounds [4]
    # (xmin, xmax, ymin, ymax); bc [4] (x-min, y-min, x-max, y-max: 0 vacuum,
    # 1 reflective); edc_mu / edc_w Larsen-EDC quadrature (cos theta and
    # azimuthal x polar weight per angle pair); and either fsr_box [R][4]
    # (xmin, xmax, ymin, ymax of the lattice cell holding each FSR) or a
    # fixed mesh: fsr_cell [R] with widths_x, widths_y.
    cmfd_geometry: Optional[Dict[str, np.ndarray]] = None
    # Extruded 3D lattices: each track's start and end points [T][6]
    # (x0, y0, z0, x1, y1, z1), float64
    track_ends: Optional[np.ndarray] = None

    @property
    def fluxes_per_track(self) -> int:
        """Angular flux values per track direction (``Solver.cpp:432-446``)."""
        return self.num_groups * self.num_polar_half

    @property
    def integrations_per_sweep(self) -> int:
        """Segment x group x polar integrations of one sweep, both
        directions: 2 * F * S, the count of ``Solver.cpp:1901``."""
        return 2 * self.fluxes_per_track * self.num_segments

    def fissile_materials(self) -> np.ndarray:
        return (self.nu_sigma_f.reshape(self.num_materials, -1) > 0).any(axis=1)

    def num_fissionable_fsrs(self) -> int:
        return int(self.fissile_materials()[self.fsr_mat].sum())

    def contiguous(self) -> "Problem":
        for name, dt in _ARRAY_DTYPES.items():
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=dt))
        if self.fixed_sources is not None:
            self.fixed_sources = np.ascontiguousarray(self.fixed_sources, np.float32)
        if self.linear_source is not None:
            self.linear_source = {k: np.ascontiguousarray(v, LS_DTYPES.get(k, v.dtype))
                                  for k, v in self.linear_source.items()}
        return self

    def validate(self, deep: bool = True) -> None:
        """Host-side checks of every packed index, raising ``ValueError``
        the way OpenMOC's ``log_printf(ERROR, ...)`` raises.  deep=False
        checks the array sizes and dimensions only (the C ABI checks every
        element again on upload, the segments on the device)."""
        G, R, T, S, M = (self.num_groups, self.num_fsrs, self.num_tracks,
                         self.num_segments, self.num_materials)
        A, Ph = self.num_angles, self.num_polar_half
        shapes = {
            "seg_len": S, "seg_fsr": S, "seg_off": T + 1, "track_ang": T,
            "next": 2 * T, "flags": T, "weights": A * Ph, "inv_sin": A * Ph,
            "sigma_t": M * G, "sigma_s": M * G * G, "nu_sigma_f": M * G,
            "chi": M * G, "fsr_mat": R, "fsr_vol": R,
        }
        for name, n in shapes.items():
            a = getattr(self, name)
            if a.size != n:
                raise ValueError(f"{name} has {a.size} entries, expected {n}")
        if G < 1 or Ph < 1 or R < 1 or T < 1 or M < 1:
            raise ValueError("empty problem dimension")
        if self.fixed_sources is not None and self.fixed_sources.size != R * G:
            raise ValueError("fixed_sources must hold num_fsrs * num_groups")
        if not deep:
            return
        if self.seg_off[0] != 0 or self.seg_off[-1] != S:
            raise ValueError("seg_off must start at 0 and end at num_segments")
        if np.any(np.diff(self.seg_off) < 0):
            raise ValueError("seg_off must be non-decreasing")
        if S and (self.seg_fsr.min() < 0 or self.seg_fsr.max() >= R):
            raise ValueError("segment FSR id out of range")
        if S and not np.all(np.isfinite(self.seg_len)):
            raise ValueError("non-finite segment length")
        if S and self.seg_len.min() < 0:
            raise ValueError("negative segment length")
        if self.next.min() < 0 or self.next.max() >= T:
            raise ValueError("next-track index out of range")
        if self.track_ang.min() < 0 or self.track_ang.max() >= A:
            raise ValueError("track angle index out of range")
        if self.fsr_mat.min() < 0 or self.fsr_mat.max() >= M:
            raise ValueError("FSR material index out of range")
        for name in ("sigma_t", "sigma_s", "nu_sigma_f", "chi", "fsr_vol",
                     "weights", "inv_sin"):
            if not np.all(np.isfinite(getattr(self, name))):
                raise ValueError(f"non-finite values in {name}")
        if self.sigma_t.min() <= 0:
            raise ValueError("sigma_t must be positive")
        if self.fixed_sources is not None and self.fixed_sources.size != R * G:
            raise ValueError("fixed_sources must hold num_fsrs * num_groups")

    def with_xs(self, sigma_t, sigma_s, nu_sigma_f, chi) -> "Problem":
        """A copy sharing the tracks but with other cross sections (same
        materials; the group count follows the new arrays)."""
        p = Problem(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        p.sigma_t = np.ascontiguousarray(sigma_t, np.float32).ravel()
        p.sigma_s = np.ascontiguousarray(sigma_s, np.float32).ravel()
        p.nu_sigma_f = np.ascontiguousarray(nu_sigma_f, np.float32).ravel()
        p.chi = np.ascontiguousarray(chi, np.float32).ravel()
        if p.sigma_t.size % p.num_materials:
            raise ValueError("sigma_t must hold num_materials x groups values")
        p.num_groups = p.sigma_t.size // p.num_materials
        p.fixed_sources = None
        p.meta = dict(self.meta)
        p.validate()
        return p


def instances(problem: Problem, xs_sets) -> Problem:
    """One problem holding K cross-section sets over ``problem``'s tracks
    and FSRs, for ``GB300Solver.setInstances(K)``: the groups of the K sets
    side by side (wide group k * G + g), the scattering matrix block
    diagonal.  ``xs_sets`` is a list of (sigma_t, sigma_s, nu_sigma_f, chi)
    in the layout of ``Problem`` (the same materials, G groups each), e.g.
    from ``lattice.pack_materials``."""
    K = len(xs_sets)
    M = problem.num_materials
    st0 = np.asarray(xs_sets[0][0], np.float32).reshape(M, -1)
    G = st0.shape[1]
    W = K * G
    st = np.zeros((M, W), np.float32)
    nf = np.zeros((M, W), np.float32)
    ch = np.zeros((M, W), np.float32)
    ss = np.zeros((M, W, W), np.float32)
    for k, (a, b, c, d) in enumerate(xs_sets):
        sl = slice(k * G, (k + 1) * G)
        st[:, sl] = np.asarray(a, np.float32).reshape(M, G)
        ss[:, sl, sl] = np.asarray(b, np.float32).reshape(M, G, G)
        nf[:, sl] = np.asarray(c, np.float32).reshape(M, G)
        ch[:, sl] = np.asarray(d, np.float32).reshape(M, G)
    wide = problem.with_xs(st, ss, nf, ch)
    wide.meta = dict(problem.meta, instances=K, instance_groups=G)
    return wide


def load_packed(base: str) -> Tuple[Problem, Dict[str, float], Dict[str, np.ndarray]]:
    """Reads ``<base>.json`` + ``<base>.bin`` (the format written by
    tests/golden/make_fixtures.cpp).  Returns the problem, the scalar
    entries and every array entry (problem arrays included)."""
    with open(base + ".json") as f:
        meta = json.load(f)
    raw = np.fromfile(base + ".bin", dtype=np.uint8)
    arrays = {}
    for name, d in meta["arrays"].items():
        dt = np.dtype(d["dtype"])
        n = d["count"]
        off = d["offset"]
        arrays[name] = raw[off:off + n * dt.itemsize].view(dt).copy()
    sc = meta["scalars"]
    p = Problem(
        num_groups=int(sc["num_groups"]),
        num_polar_half=int(sc["num_polar_half"]),
        num_angles=int(sc["num_angles"]),
        num_materials=int(sc["num_materials"]),
        num_fsrs=int(sc["num_fsrs"]),
        num_tracks=int(sc["num_tracks"]),
        num_segments=int(sc["num_segments"]),
        solve_3d=int(sc["solve_3d"]),
        **{k: arrays[k] for k in _ARRAY_DTYPES},
    )
    for key in ("fixed_sources", "fixed_source"):
        if key in arrays:
            p.fixed_sources = arrays[key]
    if "ls_seg_x" in arrays:
        p.linear_source = {k: arrays["ls_" + k]
                           for k in LS_KEYS + LS_KEYS_3D + ("centroid",)
                           if "ls_" + k in arrays}
    if "cm_end_face" in arrays:
        p.cmfd_geometry = {k[3:]: v for k, v in arrays.items() if k.startswith("cm_")}
    p.meta = dict(sc)
    return p.contiguous(), sc, arrays


def save_packed(base: str, p: Problem, extra_scalars=None, extra_arrays=None) -> None:
    """Writes a problem in the same .json + .bin format."""
    arrays = {k: getattr(p, k) for k in _ARRAY_DTYPES}
    if p.fixed_sources is not None:
        arrays["fixed_sources"] = p.fixed_sources
    if p.linear_source is not None:
        for k, v in p.linear_source.items():
            arrays["ls_" + k] = np.ascontiguousarray(v, LS_DTYPES.get(k, v.dtype))
    if p.cmfd_geometry is not None:
        for k, v in p.cmfd_geometry.items():
            arrays["cm_" + k] = np.ascontiguousarray(v)
    if extra_arrays:
        arrays.update(extra_arrays)
    scalars = {k: getattr(p, k) for k in (
        "num_groups", "num_polar_half", "num_angles", "num_materials",
        "num_fsrs", "num_tracks", "num_segments", "solve_3d")}
    if extra_scalars:
        scalars.update(extra_scalars)
    entries = {}
    off = 0
    os.makedirs(os.path.dirname(os.path.abspath(base)), exist_ok=True)
    with open(base + ".bin", "wb") as f:
        for name, a in arrays.items():
            a = np.ascontiguousarray(a)
            pad = (-off) % 16
            f.write(b"\0" * pad)
            off += pad
            entries[name] = {"dtype": a.dtype.str.lstrip("<|="), "offset": off,
                             "count": int(a.size)}
            f.write(a.tobytes())
            off += a.nbytes
    with open(base + ".json", "w") as f:
        json.dump({"precision": "f32", "arrays": entries,
                   "scalars": {k: float(v) for k, v in scalars.items()}}, f,
                  indent=1)
