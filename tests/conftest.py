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
# Linear-source solves (CPULSSolver): the reference's own
# test_2d_gradient_linear_source and test_fixed_linear_source replicas, an
# eigenvalue pin cell and a computeSource lattice.
LS_CASES = ["grad2d_ls", "fixls_c5g7", "pin7_ls", "src3_ls"]
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
                                 "ls_ang_wgt", "ls_pol_sin", "ls_pol_wgt")}
    if "fixed_source_xy" in arr:
        d["fixed_xy"] = arr["fixed_source_xy"]
    return d
