"""ctypes binding of libopenmoc_gb300.so (the C ABI of
``include/openmoc_gb300.h``).

The library is loaded from ``openmoc_gb300/_lib`` (built in-tree by
``openmoc_gb300.build``).  There is no fallback: if the library is missing
or cannot be loaded, :func:`lib` raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

MOC_OK = 0
MOC_ERR_ARG = -1
MOC_ERR_UNSUPPORTED = -5
ERRORS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "wrong call order",
    -4: "device memory exhausted",
    -5: "unsupported",
    -6: "device wait timed out",
}


class Dims(C.Structure):
    _fields_ = [
        ("num_groups", C.c_int32),
        ("num_polar_half", C.c_int32),
        ("num_angles", C.c_int32),
        ("num_materials", C.c_int32),
        ("num_fsrs", C.c_int64),
        ("num_tracks", C.c_int64),
        ("num_segments", C.c_int64),
        ("solve_3d", C.c_int32),
        ("device", C.c_int32),
    ]


class LSGeometry(C.Structure):
    """moc_ls_geometry: the linear-source arrays (pointers; seg_z and
    pol_cos for explicit 3D tracks, else null)."""
    _fields_ = [("seg_x", C.c_void_p), ("seg_y", C.c_void_p),
                ("ang_dir", C.c_void_p), ("ang_wgt", C.c_void_p),
                ("pol_sin", C.c_void_p), ("pol_wgt", C.c_void_p),
                ("seg_z", C.c_void_p), ("pol_cos", C.c_void_p)]


class OtfTracks(C.Structure):
    """moc_otf_tracks: the on-the-fly description of extruded 3D tracks."""
    _fields_ = [("num_radial_tracks", C.c_int64), ("num_radial_segments", C.c_int64),
                ("trk", C.c_void_p), ("trk_f", C.c_void_p), ("ang", C.c_void_p),
                ("rad_len", C.c_void_p), ("rad_fsr", C.c_void_p),
                ("rad_off", C.c_void_p), ("rad_start", C.c_void_p),
                ("rad_total", C.c_void_p), ("above_fsr", C.c_int32)]


class CmfdMesh(C.Structure):
    """moc_cmfd_mesh: the coarse mesh and settings of CMFD acceleration."""
    _fields_ = [("num_x", C.c_int32), ("num_y", C.c_int32),
                ("widths_x", C.c_void_p), ("widths_y", C.c_void_p),
                ("fsr_cell", C.c_void_p), ("track_end_face", C.c_void_p),
                ("boundary", C.c_int32 * 4), ("num_cmfd_groups", C.c_int32),
                ("group_of", C.c_void_p), ("num_edc_angles", C.c_int32),
                ("edc_mu", C.c_void_p), ("edc_weight", C.c_void_p),
                ("relaxation", C.c_double), ("sor_factor", C.c_double),
                ("flux_limiting", C.c_int32),
                ("num_unbounded_iterations", C.c_int32),
                ("solve_on_host", C.c_int32), ("k_nearest", C.c_int32),
                ("fsr_centroid", C.c_void_p), ("origin_x", C.c_double),
                ("origin_y", C.c_double)]


_P = C.c_void_p
_SIGS = {
    "moc_last_error": ([], C.c_char_p),
    "moc_version": ([], C.c_char_p),
    "moc_release_cached_memory": ([], C.c_int),
    "moc_create": ([C.POINTER(Dims), C.POINTER(C.c_void_p)], C.c_int),
    "moc_destroy": ([_P], C.c_int),
    "moc_upload_tracks": ([_P, _P, _P, _P, _P, _P, _P], C.c_int),
    "moc_upload_quadrature": ([_P, _P, _P], C.c_int),
    "moc_upload_materials": ([_P, _P, _P, _P, _P], C.c_int),
    "moc_upload_sigma_f": ([_P, _P], C.c_int),
    "moc_upload_fsrs": ([_P, _P, _P], C.c_int),
    "moc_set_fixed_sources": ([_P, _P], C.c_int),
    "moc_set_convergence_threshold": ([_P, C.c_double], C.c_int),
    "moc_set_exponential": ([_P, C.c_int], C.c_int),
    "moc_get_exponential": ([_P, C.POINTER(C.c_int)], C.c_int),
    "moc_set_autotune": ([_P, C.c_int], C.c_int),
    "moc_autotune": ([_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)],
                     C.c_int),
    "moc_get_tuning_log": ([_P, _P, _P, _P, _P, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "moc_set_sweep_shape": ([_P, C.c_int, C.c_int], C.c_int),
    "moc_get_sweep_shape": ([_P, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
    "moc_set_iterations_per_sync": ([_P, C.c_int], C.c_int),
    "moc_set_source_kernel": ([_P, C.c_int], C.c_int),
    "moc_get_source_kernel": ([_P, C.POINTER(C.c_int)], C.c_int),
    "moc_set_tensor_wait_limit": ([_P, C.c_int64], C.c_int),
    "moc_compute_eigenvalue": ([_P, C.c_int, C.c_int], C.c_int),
    "moc_compute_source": ([_P, C.c_int, C.c_double, C.c_int], C.c_int),
    "moc_compute_flux": ([_P, C.c_int, C.c_int], C.c_int),
    "moc_get_keff": ([_P, C.POINTER(C.c_double)], C.c_int),
    "moc_get_num_iterations": ([_P, C.POINTER(C.c_int)], C.c_int),
    "moc_get_residual": ([_P, C.POINTER(C.c_double)], C.c_int),
    "moc_get_fluxes": ([_P, _P, C.c_int64], C.c_int),
    "moc_set_fluxes": ([_P, _P, C.c_int64], C.c_int),
    "moc_get_sweep_time": ([_P, C.POINTER(C.c_double), C.POINTER(C.c_int64)], C.c_int),
    "moc_zero_track_fluxes": ([_P], C.c_int),
    "moc_flatten_fsr_fluxes": ([_P, C.c_float], C.c_int),
    "moc_flatten_fsr_fluxes_chi": ([_P, C.c_int], C.c_int),
    "moc_store_fsr_fluxes": ([_P], C.c_int),
    "moc_normalize_fluxes": ([_P, C.POINTER(C.c_double)], C.c_int),
    "moc_compute_fsr_sources": ([_P, C.c_int], C.c_int),
    "moc_transport_sweep": ([_P], C.c_int),
    "moc_add_source_to_scalar_flux": ([_P], C.c_int),
    "moc_compute_keff": ([_P], C.c_int),
    "moc_compute_residual": ([_P, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "moc_set_keff": ([_P, C.c_double], C.c_int),
    "moc_compute_fsr_fission_rates": ([_P, _P, C.c_int64, C.c_int], C.c_int),
    "moc_get_reduced_sources": ([_P, _P, C.c_int64], C.c_int),
    "moc_get_old_fluxes": ([_P, _P, C.c_int64], C.c_int),
    "moc_set_old_fluxes": ([_P, _P, C.c_int64], C.c_int),
    "moc_get_start_flux": ([_P, _P, C.c_int64], C.c_int),
    "moc_set_start_flux": ([_P, _P, C.c_int64], C.c_int),
    "moc_get_launch_count": ([_P, C.POINTER(C.c_int64)], C.c_int),
    "moc_bench_iterations": ([_P, C.c_int, C.c_int, C.c_int, _P, _P], C.c_int),
    "moc_eval_attenuation": ([_P, C.c_int, _P, _P, C.c_int64], C.c_int),
    "moc_fission_source_total_noalloc": ([_P, C.c_int64, _P, C.c_int32, _P, _P,
                                          C.c_int64, C.c_int32, _P, _P], C.c_int),
    "moc_set_linear_source": ([_P, C.POINTER(LSGeometry)], C.c_int),
    "moc_get_linear_source": ([_P, C.POINTER(C.c_int), C.POINTER(C.c_int64)], C.c_int),
    "moc_get_flux_moments": ([_P, _P, C.c_int64], C.c_int),
    "moc_set_flux_moments": ([_P, _P, C.c_int64], C.c_int),
    "moc_get_source_moments": ([_P, _P, C.c_int64], C.c_int),
    "moc_set_fixed_source_moments": ([_P, _P, C.c_int64], C.c_int),
    "moc_get_linear_expansion": ([_P, _P, _P], C.c_int),
    "moc_set_negative_fluxes_allowed": ([_P, C.c_int], C.c_int),
    "moc_set_keff_from_neutron_balance": ([_P, C.c_int], C.c_int),
    "moc_set_instances": ([_P, C.c_int], C.c_int),
    "moc_get_instance_keffs": ([_P, _P, C.c_int], C.c_int),
    "moc_set_transport_stabilization": ([_P, C.c_int, C.c_double, C.c_int], C.c_int),
    "moc_compute_stabilizing_flux": ([_P], C.c_int),
    "moc_stabilize_flux": ([_P], C.c_int),
    "moc_compute_fsr_fission_sources": ([_P], C.c_int),
    "moc_compute_fsr_scatter_sources": ([_P], C.c_int),
    "moc_set_otf_tracks": ([_P, C.POINTER(OtfTracks)], C.c_int),
    "moc_get_otf_tracks": ([_P, C.POINTER(C.c_int)], C.c_int),
    "moc_set_cmfd": ([_P, C.POINTER(CmfdMesh)], C.c_int),
    "moc_get_cmfd_info": ([_P, C.POINTER(C.c_int), C.POINTER(C.c_double),
                           C.POINTER(C.c_int), C.POINTER(C.c_int),
                           C.POINTER(C.c_double), C.POINTER(C.c_int)], C.c_int),
    "moc_get_cmfd_fluxes": ([_P, _P, _P, C.c_int64], C.c_int),
}

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Loads libopenmoc_gb300.so (building it first if it is absent and
    ``build_if_missing``).  Raises RuntimeError when it cannot be loaded."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: run openmoc_gb300.build")
            _build.build()
        try:
            L = C.CDLL(path)
        except OSError as e:
            raise RuntimeError(f"cannot load {path}: {e}") from e
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return L


def exported_symbols():
    return list(_SIGS)


class MOCError(RuntimeError):
    """Raised for every non-zero status of the C ABI (OpenMOC maps its
    ERROR log level to a Python RuntimeError the same way)."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{ERRORS.get(status, 'error')} ({status}): {message}")


def check(status: int) -> None:
    if status != MOC_OK:
        msg = lib().moc_last_error().decode(errors="replace")
        raise MOCError(status, msg)
