import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# Cases produced by tests/golden/make_fixtures.cpp from OpenMOC itself:
# eigenvalue solves, and fixed-source solves (computeSource, computeFlux).
CASES = ["pin_c5g7", "pin_70g", "pin7_synth", "lat3_g2_vac", "lat2_g16"]
SRC_CASES = ["src3_g7", "flux3_g7"]
# Explicit 3D tracks (TrackGenerator3D with EXPLICIT_3D segments).
CASES_3D = ["pin3d_g7"]
# keff from the neutron balance (Solver::setKeffFromNeutronBalance); its
# probe also holds the fission / scattering source hooks.
BALANCE_CASES = ["lat3_bal"]
# Transport stabilization (Solver::stabilizeTransport): YAMAMOTO, GLOBAL,
# DIAGONAL (a moderator with negative within-group scattering).
STAB_CASES = ["pin7_stab_y", "pin7_stab_g", "lat3_stab_d"]
# Linear-source solves (CPULSSolver): the reference's own
# test_2d_gradient_linear_source and test_fixed_linear_source replicas, an
# eigenvalue pin cell and a computeSource lattice.
LS_CASES = ["grad2d_ls", "fixls_c5g7", "pin7_ls", "src3_ls"]
# CPULSSolver on explicit 3D tracks (x, y and z moments)
LS_CASES_3D = ["pin3d_ls"]
LS_PROBE_CASES = ["grad2d_ls", "pin7_ls"]
# CMFD-accelerated eigenvalue solves (Geometry::setCmfd) and the coarse
# group structure each case set (None: one coarse group per group).
CMFD_CASES = {"cmfd_lat3": [[1, 2, 3], [4, 5, 6, 7]], "cmfd_lat5_vac": None,
              "cmfd_lat3_ls": [[1, 2, 3], [4, 5, 6, 7]],
              "cmfd_lat3_k3": [[1, 2, 3], [4, 5, 6, 7]]}
# SOR factor each case set (the linear-source case runs CPULSSolver)
CMFD_SOR = {"cmfd_lat3": 1.5, "cmfd_lat5_vac": 1.5, "cmfd_lat3_ls": 1.0,
            "cmfd_lat3_k3": 1.5}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_case(name, precision="f32"):
    from openmoc_gb300.problem import load_packed
    return load_packed(os.path.join(GOLDEN, f"{name}_{precision}"))


def ls_arrays(arr):
    """The linear-source geometry of a fixture (and its fixed source moments,
    if any) under the names of the oracle and of the solver API."""
    d = {k[3:]: arr[k] for k in ("ls_seg_x", "ls_seg_y", "ls_ang_dir",
                                 "ls_ang_wgt", "ls_pol_sin", "ls_pol_wgt",
                                 "ls_seg_z", "ls_pol_cos") if k in arr}
    if "fixed_source_xy" in arr:
        d["fixed_xy"] = arr["fixed_source_xy"]
    return d


def load_openmoc_config_golden(config):
    """OpenMOC's FP64 CPUSolver on a benchmark configuration after a fixed
    number of source iterations (tests/golden/make_config_goldens.sh):
    track checksums, keff, per-group flux sums and a sample of FSR fluxes."""
    import json
    with open(os.path.join(GOLDEN, f"openmoc_{config}_f64.json")) as f:
        return json.load(f)


def track_checksum(a):
    """The order-sensitive checksum oracle/openmoc_run.cpp writes: the sum
    over i of (word_i + 1) * (2 i + 1) mod 2^64, word_i the i-th element's
    bytes as a little-endian unsigned integer."""
    import numpy as np
    a = np.ascontiguousarray(a)
    words = a.view({1: np.uint8, 4: np.uint32, 8: np.uint64}[a.itemsize]).astype(np.uint64)
    i = np.arange(a.size, dtype=np.uint64)
    return int(np.sum((words + np.uint64(1)) * (np.uint64(2) * i + np.uint64(1)),
                      dtype=np.uint64))


def quantised_sums(a, bits):
    """The plain and the (i mod 1009 + 1)-weighted sum, mod 2^64, of
    q_i = floor(a_i * 2^bits + 1/2): the exact integer sums
    oracle/openmoc_run.cpp writes for segment lengths and volumes."""
    import numpy as np
    q = np.floor(np.asarray(a, np.float64) * 2.0 ** bits + 0.5).astype(np.int64)
    q = q.view(np.uint64)
    w = (np.arange(q.size) % 1009 + 1).astype(np.uint64)
    return int(np.sum(q, dtype=np.uint64)), int(np.sum(w * q, dtype=np.uint64))


def wrapped_difference(a, b):
    """a - b for two sums kept mod 2^64, as a signed integer."""
    d = (int(a) - int(b)) % (1 << 64)
    return d - (1 << 64) if d >= (1 << 63) else d


def errors_against_golden(keff, flux, golden):
    """|keff - keff_ref|, the largest relative error over the golden's flux
    sample and over its per-group flux sums."""
    import numpy as np
    flux = np.asarray(flux, np.float64).ravel()
    G = int(golden["num_groups"])
    idx = np.asarray(golden["flux_sample_index"], np.int64)
    ref = np.asarray(golden["flux_sample"], np.float64)
    sums = flux.reshape(-1, G).sum(axis=0)
    ref_sums = np.asarray(golden["group_flux_sums"], np.float64)
    return (abs(keff - golden["keff"]),
            float(np.max(np.abs(flux[idx] - ref) / np.abs(ref))),
            float(np.max(np.abs(sums - ref_sums) / np.abs(ref_sums))))
