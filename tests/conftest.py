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


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_case(name, precision="f32"):
    from openmoc_gb300.problem import load_packed
    return load_packed(os.path.join(GOLDEN, f"{name}_{precision}"))
