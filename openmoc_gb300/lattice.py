"""Pin-lattice workloads: tracks and segments from the library's own 2D
track generator (``include/openmoc_gb300_lattice.h``) plus seeded synthetic
cross sections, packed as a :class:`~openmoc_gb300.problem.Problem`.

The named builders are the benchmark problems:

* :func:`pin_cell` -- one pin (r = 0.54 cm, pitch 1.26 cm), fuel in 3
  equal-area rings x 8 sectors, moderator in 8 sectors, all reflective;
* :func:`assembly_17x17` -- 17 x 17 pins at 1.26 cm with the 25 water-filled
  guide-tube positions of a standard PWR assembly, reflective;
* :func:`core_51x51` -- 3 x 3 such lattices (51 x 51 pins), three fuel
  cross-section sets in a checkerboard of assemblies, vacuum on +x and +y,
  reflective on -x and -y;
* :func:`lattice` -- any n x n lattice of that pin.

Cross sections come from ``moc_synthetic_xs`` (construction documented in
``openmoc_gb300/csrc/synthetic_xs.h``) with seed ``0xC0FFEE + config``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _native
from .problem import Problem

VACUUM, REFLECTIVE = 0, 1
SEED = 0xC0FFEE

# Guide-tube positions of a 17 x 17 PWR assembly, (row, col) from the top
# left corner (24 guide tubes and the central instrument tube).
GUIDE_TUBES_17x17 = [
    (2, 5), (2, 8), (2, 11), (3, 3), (3, 13),
    (5, 2), (5, 5), (5, 8), (5, 11), (5, 14),
    (8, 2), (8, 5), (8, 8), (8, 11), (8, 14),
    (11, 2), (11, 5), (11, 8), (11, 11), (11, 14),
    (13, 3), (13, 13), (14, 5), (14, 8), (14, 11),
]


class _Spec(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("pitch", C.c_double),
        ("pin_radius", C.c_double), ("fuel_rings", C.c_int32),
        ("fuel_sectors", C.c_int32), ("mod_sectors", C.c_int32),
        ("bc", C.c_int32 * 4), ("num_azim", C.c_int32), ("spacing", C.c_double),
        ("num_polar", C.c_int32), ("moderator_material", C.c_int32),
        ("num_threads", C.c_int32), ("pin_material", C.c_void_p),
    ]


_host_library = None


def use_host_library(path: str) -> None:
    """Binds the track generator and the cross-section builder to a
    host-only build of ``csrc/lattice.cpp`` at ``path`` (the same
    ``moc_lattice_*`` / ``moc_synthetic_xs`` entry points, no CUDA code)
    instead of libopenmoc_gb300.so, for processes that must not load the GPU
    library.  Device ray tracing (``device=``) is then unavailable."""
    global _host_library
    _host_library = C.CDLL(path)


def _lib():
    L = _native.lib() if _host_library is None else _host_library
    if not getattr(L, "_lattice_sigs", False):
        L.moc_lattice_generate.argtypes = [C.POINTER(_Spec), C.POINTER(C.c_void_p)]
        L.moc_lattice_generate.restype = C.c_int
        L.moc_lattice_sizes.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 3 + \
            [C.POINTER(C.c_int32)] * 3
        L.moc_lattice_sizes.restype = C.c_int
        L.moc_lattice_export.argtypes = [C.c_void_p] + [C.c_void_p] * 10
        L.moc_lattice_export.restype = C.c_int
        L.moc_lattice_extrude.argtypes = [C.c_void_p, C.c_double, C.c_double,
                                          C.c_double, C.c_int32, C.c_int32,
                                          C.POINTER(C.c_void_p)]
        L.moc_lattice_extrude.restype = C.c_int
        if hasattr(L, "moc_lattice_generate_device"):
            L.moc_lattice_generate_device.argtypes = [C.POINTER(_Spec), C.c_int32,
                                                      C.POINTER(C.c_void_p)]
            L.moc_lattice_generate_device.restype = C.c_int
        L.moc_lattice_otf_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_int64),
                                            C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
        L.moc_lattice_otf_sizes.restype = C.c_int
        L.moc_lattice_export_otf.argtypes = [C.c_void_p] + [C.c_void_p] * 8
        L.moc_lattice_export_otf.restype = C.c_int
        L.moc_lattice_export_ends3d.argtypes = [C.c_void_p, C.c_void_p]
        L.moc_lattice_export_ends3d.restype = C.c_int
        L.moc_lattice_export_ls.argtypes = [C.c_void_p] + [C.c_void_p] * 7
        L.moc_lattice_export_ls.restype = C.c_int
        L.moc_lattice_export_ls3d.argtypes = [C.c_void_p] + [C.c_void_p] * 9
        L.moc_lattice_export_ls3d.restype = C.c_int
        L.moc_lattice_export_cmfd.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        L.moc_lattice_export_cmfd.restype = C.c_int
        L.moc_lattice_destroy.argtypes = [C.c_void_p]
        L.moc_lattice_destroy.restype = C.c_int
        L.moc_lattice_last_error.restype = C.c_char_p
        L.moc_synthetic_xs.argtypes = [C.c_uint64, C.c_int32, C.c_int32, C.c_uint64,
                                       C.c_double] + [C.c_void_p] * 5
        L.moc_synthetic_xs.restype = C.c_int
        L._lattice_sigs = True
    return L


@dataclass
class MaterialXS:
    sigma_t: np.ndarray      # [G]
    sigma_s: np.ndarray      # [G, G] origin-major: [orig, dest]
    nu_sigma_f: np.ndarray   # [G]
    sigma_f: np.ndarray      # [G]
    chi: np.ndarray          # [G]

    @property
    def num_groups(self) -> int:
        return self.sigma_t.size


def synthetic_xs(seed: int, num_groups: int, fissile: bool,
                 perturb_seed: int = 0, perturb_sigma: float = 0.0) -> MaterialXS:
    G = int(num_groups)
    st = np.zeros(G)
    ss = np.zeros(G * G)
    nf = np.zeros(G)
    sf = np.zeros(G)
    ch = np.zeros(G)
    rc = _lib().moc_synthetic_xs(seed, G, int(fissile), perturb_seed, perturb_sigma,
                                 st.ctypes.data, ss.ctypes.data, nf.ctypes.data,
                                 sf.ctypes.data, ch.ctypes.data)
    if rc:
        raise RuntimeError(_lib().moc_lattice_last_error().decode())
    return MaterialXS(st, ss.reshape(G, G), nf, sf, ch)


def pack_materials(mats: Sequence[MaterialXS]):
    """Material arrays in the C ABI layout (float32; scattering
    destination-major, as Material::getSigmaS stores it)."""
    G = mats[0].num_groups
    sigma_t = np.stack([m.sigma_t for m in mats]).astype(np.float32)
    sigma_s = np.stack([m.sigma_s.T for m in mats]).astype(np.float32)
    nu_sigma_f = np.stack([m.nu_sigma_f for m in mats]).astype(np.float32)
    chi = np.stack([m.chi for m in mats]).astype(np.float32)
    # Material::setSigmaT clamps |sigma_t| < 1e-10 (src/Material.cpp:628-650)
    sigma_t = np.where(np.abs(sigma_t) < 1e-10, np.float32(1e-10), sigma_t)
    assert sigma_s.shape == (len(mats), G, G)
    return sigma_t.ravel(), sigma_s.ravel(), nu_sigma_f.ravel(), chi.ravel()


def lattice(nx: int, ny: int, pin_material: np.ndarray, materials: Sequence[MaterialXS],
            moderator_material: int, *, num_azim: int, spacing: float,
            pitch: float = 1.26, pin_radius: float = 0.54, fuel_rings: int = 3,
            fuel_sectors: int = 8, mod_sectors: int = 8, num_polar: int = 6,
            bc=(REFLECTIVE, REFLECTIVE, REFLECTIVE, REFLECTIVE),
            num_threads: int = 0, extrude: Optional[dict] = None,
            linear_source: bool = False, device: Optional[int] = None) -> Problem:
    """Tracks, segments and cross sections of an nx x ny pin lattice.
    ``pin_material[row, col]`` (row 0 = top) is the material inside each
    pin; ``bc`` is (xmin, xmax, ymin, ymax).  ``extrude`` = dict(height,
    fuel_height, z_spacing, num_polar) turns it into explicit 3D tracks of
    the lattice extruded axially (moderator above fuel_height, vacuum at
    bottom and top; ``num_polar`` Gauss-Legendre polar angles).
    ``linear_source`` also exports the linear-source geometry: segment
    starts relative to the FSR centroids and the angle data (with z starts
    and cos theta for extruded 3D tracks), as ``Problem.linear_source``.
    ``device`` ray-traces on that CUDA device (the same segments and FSR
    ids; moc_lattice_generate_device)."""
    L = _lib()
    pm = np.ascontiguousarray(np.asarray(pin_material, np.int32).reshape(ny, nx))
    spec = _Spec(nx, ny, pitch, pin_radius, fuel_rings, fuel_sectors, mod_sectors,
                 (C.c_int32 * 4)(*bc), num_azim, spacing, num_polar,
                 moderator_material, num_threads, pm.ctypes.data)
    h = C.c_void_p()
    rc = (L.moc_lattice_generate(C.byref(spec), C.byref(h)) if device is None else
          L.moc_lattice_generate_device(C.byref(spec), int(device), C.byref(h)))
    if rc:
        raise RuntimeError(L.moc_lattice_last_error().decode())
    if extrude is not None:
        h3 = C.c_void_p()
        rc = L.moc_lattice_extrude(h, float(extrude["height"]),
                                   float(extrude["fuel_height"]),
                                   float(extrude["z_spacing"]),
                                   int(extrude["num_polar"]), num_threads,
                                   C.byref(h3))
        L.moc_lattice_destroy(h)
        if rc:
            raise RuntimeError(L.moc_lattice_last_error().decode())
        h = h3
    try:
        R, T, S = C.c_int64(), C.c_int64(), C.c_int64()
        A, Ph, M = C.c_int32(), C.c_int32(), C.c_int32()
        L.moc_lattice_sizes(h, C.byref(R), C.byref(T), C.byref(S), C.byref(A),
                            C.byref(Ph), C.byref(M))
        R, T, S, A, Ph = R.value, T.value, S.value, A.value, Ph.value
        arr = dict(
            seg_len=np.empty(S, np.float32), seg_fsr=np.empty(S, np.int32),
            seg_off=np.empty(T + 1, np.int64), track_ang=np.empty(T, np.int32),
            next=np.empty(2 * T, np.int64), flags=np.empty(T, np.uint8),
            weights=np.empty(A * Ph, np.float32), inv_sin=np.empty(A * Ph, np.float32),
            fsr_mat=np.empty(R, np.int32), fsr_vol=np.empty(R, np.float32))
        L.moc_lattice_export(h, *[arr[k].ctypes.data for k in (
            "seg_len", "seg_fsr", "seg_off", "track_ang", "next", "flags", "weights",
            "inv_sin", "fsr_mat", "fsr_vol")])
        otf = None
        if extrude is not None:
            T2, S2, above = C.c_int64(), C.c_int64(), C.c_int32()
            if L.moc_lattice_otf_sizes(h, C.byref(T2), C.byref(S2), C.byref(above)):
                raise RuntimeError(L.moc_lattice_last_error().decode())
            T2, S2 = T2.value, S2.value
            otf = dict(trk=np.empty(4 * T, np.int32), trk_f=np.empty(4 * T, np.float32),
                       ang=np.empty(4 * A, np.float32),
                       rad_len=np.empty(S2, np.float32), rad_fsr=np.empty(S2, np.int32),
                       rad_off=np.empty(T2 + 1, np.int64),
                       rad_start=np.empty(S2, np.float32),
                       rad_total=np.empty(T2, np.float32),
                       above_fsr=np.array([above.value], np.int32))
            if L.moc_lattice_export_otf(h, *[otf[k].ctypes.data for k in (
                    "trk", "trk_f", "ang", "rad_len", "rad_fsr", "rad_off",
                    "rad_start", "rad_total")]):
                raise RuntimeError(L.moc_lattice_last_error().decode())
            ends = np.empty((T, 6), np.float64)
            if L.moc_lattice_export_ends3d(h, ends.ctypes.data):
                raise RuntimeError(L.moc_lattice_last_error().decode())
        ls = None
        if linear_source and extrude is not None:
            ls = dict(seg_x=np.empty(S, np.float32), seg_y=np.empty(S, np.float32),
                      seg_z=np.empty(S, np.float32), centroid=np.empty(3 * R),
                      ang_dir=np.empty(2 * A), ang_wgt=np.empty(A),
                      pol_sin=np.empty(A), pol_cos=np.empty(A), pol_wgt=np.empty(A))
            if L.moc_lattice_export_ls3d(h, *[ls[k].ctypes.data for k in (
                    "seg_x", "seg_y", "seg_z", "centroid", "ang_dir", "ang_wgt",
                    "pol_sin", "pol_cos", "pol_wgt")]):
                raise RuntimeError(L.moc_lattice_last_error().decode())
        elif linear_source:
            ls = dict(seg_x=np.empty(S, np.float32), seg_y=np.empty(S, np.float32),
                      centroid=np.empty(2 * R), ang_dir=np.empty(2 * A),
                      ang_wgt=np.empty(A), pol_sin=np.empty(A * Ph),
                      pol_wgt=np.empty(A * Ph))
            if L.moc_lattice_export_ls(h, *[ls[k].ctypes.data for k in (
                    "seg_x", "seg_y", "centroid", "ang_dir", "ang_wgt", "pol_sin",
                    "pol_wgt")]):
                raise RuntimeError(L.moc_lattice_last_error().decode())
        cm = None
        if extrude is None:
            cm = dict(fsr_box=np.empty(4 * R), end_face=np.empty(2 * T, np.int8),
                      edc_mu=np.empty(A * Ph), edc_w=np.empty(A * Ph),
                      bounds=np.empty(4), fsr_centroid=np.empty(2 * R))
            if L.moc_lattice_export_cmfd(h, *[cm[k].ctypes.data for k in (
                    "fsr_box", "end_face", "edc_mu", "edc_w", "bounds",
                    "fsr_centroid")]):
                raise RuntimeError(L.moc_lattice_last_error().decode())
            cm["fsr_box"] = cm["fsr_box"].reshape(R, 4)
            # (x-min, y-min, x-max, y-max) from bc = (xmin, xmax, ymin, ymax)
            cm["bc"] = np.array([bc[0], bc[2], bc[1], bc[3]], np.int32)
    finally:
        L.moc_lattice_destroy(h)
    st, ss, nf, ch = pack_materials(materials)
    G = materials[0].num_groups
    p = Problem(num_groups=G, num_polar_half=Ph, num_angles=A,
                num_materials=len(materials), num_fsrs=R, num_tracks=T,
                num_segments=S, solve_3d=0 if extrude is None else 1,
                sigma_t=st, sigma_s=ss, nu_sigma_f=nf,
                chi=ch, **arr)
    p.linear_source = ls
    p.otf = otf
    p.cmfd_geometry = cm
    if extrude is not None:
        p.track_ends = ends
    p.meta = dict(nx=nx, ny=ny, num_azim=num_azim, spacing=spacing, pitch=pitch,
                  num_polar=num_polar)
    return p.contiguous()


def _fuel_mod(config: int, G: int, n_fuel: int = 1, perturb=None):
    mats = []
    for k in range(n_fuel):
        mats.append(synthetic_xs(SEED + config + k, G, True))
    mats.append(synthetic_xs(SEED + config + 1000, G, False))
    if perturb is not None:
        seed, sigma = perturb
        mats = [synthetic_xs(SEED + config + (k if k < n_fuel else 1000), G, k < n_fuel,
                             seed + k, sigma) for k in range(n_fuel + 1)]
    return mats


def pin_cell(num_groups: int = 7, num_azim: int = 32, spacing: float = 0.05,
             config: int = 0, perturb=None, linear_source: bool = False,
             device: Optional[int] = None) -> Problem:
    """One pin cell, all reflective (the 7-group pin-cell benchmark)."""
    mats = _fuel_mod(config, num_groups, 1, perturb)
    return lattice(1, 1, np.zeros((1, 1), np.int32), mats, 1,
                   num_azim=num_azim, spacing=spacing, linear_source=linear_source,
                   device=device)


def square_lattice(n: int, num_groups: int, num_azim: int, spacing: float,
                   config: int, water_pins: Optional[List] = None,
                   perturb=None, linear_source: bool = False,
                   device: Optional[int] = None) -> Problem:
    """n x n lattice of the pin; ``water_pins`` positions hold moderator."""
    mats = _fuel_mod(config, num_groups, 1, perturb)
    pm = np.zeros((n, n), np.int32)
    for (r, c) in (water_pins or []):
        pm[r, c] = 1
    return lattice(n, n, pm, mats, 1, num_azim=num_azim, spacing=spacing,
                   linear_source=linear_source, device=device)


def assembly_17x17(num_groups: int = 70, num_azim: int = 64, spacing: float = 0.05,
                   config: int = 1, perturb=None, linear_source: bool = False,
                   device: Optional[int] = None) -> Problem:
    """17 x 17 assembly with 25 water-filled guide-tube positions."""
    return square_lattice(17, num_groups, num_azim, spacing, config,
                          GUIDE_TUBES_17x17, perturb, linear_source, device)


def assembly_17x17_3d(num_groups: int = 7, num_azim: int = 16, spacing: float = 0.1,
                      num_polar: int = 6, z_spacing: float = 0.5, height: float = 20.0,
                      fuel_height: float = 16.0, config: int = 4, perturb=None,
                      linear_source: bool = False) -> Problem:
    """The 17 x 17 assembly extruded axially: the lattice for z < 16 cm,
    homogeneous moderator up to 20 cm, reflective radially, vacuum at the
    bottom and top, explicit 3D tracks (16 azimuthal, 6 polar, 0.1 cm radial,
    0.5 cm axial spacing)."""
    mats = _fuel_mod(config, num_groups, 1, perturb)
    pm = np.zeros((17, 17), np.int32)
    for (r, c) in GUIDE_TUBES_17x17:
        pm[r, c] = 1
    return lattice(17, 17, pm, mats, 1, num_azim=num_azim, spacing=spacing,
                   extrude=dict(height=height, fuel_height=fuel_height,
                                z_spacing=z_spacing, num_polar=num_polar),
                   linear_source=linear_source)


def core_51x51(num_groups: int = 7, num_azim: int = 128, spacing: float = 0.03,
               config: int = 3, device: Optional[int] = None) -> Problem:
    """3 x 3 assemblies of 17 x 17 pins, three fuel sets in a checkerboard,
    vacuum on +x and +y, reflective on -x and -y."""
    mats = _fuel_mod(config, num_groups, 3)
    pm = np.zeros((51, 51), np.int32)
    for ar in range(3):
        for ac in range(3):
            fuel = (ar + ac) % 3
            block = np.full((17, 17), fuel, np.int32)
            for (r, c) in GUIDE_TUBES_17x17:
                block[r, c] = 3
            pm[17 * ar:17 * ar + 17, 17 * ac:17 * ac + 17] = block
    return lattice(51, 51, pm, mats, 3, num_azim=num_azim, spacing=spacing,
                   bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM), device=device)
