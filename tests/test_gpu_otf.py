"""On-the-fly 3D segmentation (moc_set_otf_tracks) against the stored
explicit 3D segments of the same extruded lattice and the FP64 oracle.

The on-the-fly sweep cuts the same pieces as the explicit generator but does
not merge consecutive pieces of one region, so the two agree to rounding;
both are compared at a fixed iteration count.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

ITERS = 15


def _extruded(n=1, G=7, num_azim=8, spacing=0.1):
    from openmoc_gb300 import lattice as lat
    mats = lat._fuel_mod(4, G, 1)
    pm = np.zeros((n, n), np.int32)
    if n > 1:
        pm[n // 2, n // 2] = 1
    return lat.lattice(n, n, pm, mats, 1, num_azim=num_azim, spacing=spacing,
                       extrude=dict(height=2.0, fuel_height=1.6, z_spacing=0.4,
                                    num_polar=4))


def _solve(p, formation, shape=None):
    from openmoc_gb300 import GB300Solver
    s = GB300Solver(device=0)
    s.setSegmentFormation(formation)
    if shape:
        s.setSweepShape(*shape)
    s.setConvergenceThreshold(1e-30)
    s.setTrackGenerator(p)
    s.computeEigenvalue(ITERS, 1)
    out = s.getKeff(), s.getFluxes()
    s.close()
    return out


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-4 * np.abs(b).max())))


@pytest.mark.parametrize("n,G,shapes", [(1, 7, [None, (2, 2), (4, 1)]),
                                        (3, 16, [None, (8, 1), (4, 2)])])
def test_otf_matches_explicit_and_oracle(n, G, shapes):
    p = _extruded(n, G)
    k_e, f_e = _solve(p, "explicit")
    o = Oracle(p, "f64", num_threads=8)
    o.compute_eigenvalue(ITERS, 1, 1e-30)
    for shape in shapes:
        k_o, f_o = _solve(p, "otf", shape)
        assert abs(k_o - k_e) < 2e-6, shape
        assert _rel(f_o, f_e) < 2e-5, shape
        assert abs(k_o - o.keff) < 2e-6, shape
        assert _rel(f_o, o.phi.reshape(p.num_fsrs, G)) < 2e-5, shape


def test_otf_without_stored_segments():
    """A context given no explicit segments at all (num_segments = 0) solves
    the extruded problem from its on-the-fly description alone."""
    from openmoc_gb300 import Problem
    p = _extruded(2, 7)
    k_ref, f_ref = _solve(p, "otf")
    q = Problem(**{f: getattr(p, f) for f in p.__dataclass_fields__})
    q.seg_len = np.zeros(0, np.float32)
    q.seg_fsr = np.zeros(0, np.int32)
    q.seg_off = np.zeros(p.num_tracks + 1, np.int64)
    q.num_segments = 0
    k, f = _solve(q, "otf")
    # tallies are float atomics (and the autotuner may pick another shape):
    # equal up to summation order
    assert abs(k - k_ref) < 1e-6
    assert _rel(f, f_ref) < 1e-5


def test_otf_bad_requests_raise():
    from openmoc_gb300 import GB300Solver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300._native import MOCError
    s = GB300Solver(lat.pin_cell(7), device=0)      # 2D: no otf description
    with pytest.raises(MOCError):
        s.setSegmentFormation("otf")
    s.close()
    p = _extruded(1, 7)
    bad = dict(p.otf)
    trk = bad["trk"].copy()
    trk[4 * 3 + 2] = 10 ** 6          # crosses more radial segments than exist
    bad["trk"] = trk
    p.otf = bad
    s = GB300Solver(p, device=0)
    with pytest.raises(MOCError):
        s.setSegmentFormation("otf")
    s.close()
