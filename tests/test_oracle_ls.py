"""The linear-source oracle (oracle/moc_oracle.c, oracle_ls_*) against
OpenMOC's CPULSSolver.

Pins the restatement before it checks the CUDA path:
  * OpenMOC's own linear-source regression goldens
    (tests/test_2d_gradient_linear_source and tests/test_fixed_linear_source
    results_true.dat, copied into tests/golden/reference_results_ls.json) are
    reproduced by the fixtures OpenMOC's library wrote, and by the oracle;
  * the linear expansion matrix inverse and source constants of
    LinearExpansionGenerator, 2D and explicit 3D (pin3d_ls: x, y and z
    moments, six coefficients);
  * every linear-source fixture: iterations, keff, fluxes and flux moments
    against the FP_PRECISION=float and =double builds;
  * hook by hook from the same converged state (sources and source moments,
    sweep tallies and moments, add-source, keff, normalisation).
The reference evaluates the exponential terms with rational approximations
(src/exponentials.h:101-323, 2e-7 to 1e-6); the oracle from their
definitions.  Where the difference shows (flux moments of optically thin
regions, through F2 = 2G - F1) the bounds below say so.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, LS_CASES, LS_CASES_3D, LS_PROBE_CASES, load_case, ls_arrays
from oracle.oracle import LSOracle


def _oracle(case, precision, threads=1):
    p, sc, arr = load_case(case, precision)
    o = LSOracle(p, ls_arrays(arr), precision, num_threads=threads,
                 negative_fluxes_allowed=bool(sc.get("allow_negative", 0)))
    return o, p, sc, arr


def _solve(o, sc):
    kind = int(sc["run_kind"])
    if kind == 0:
        return o.compute_eigenvalue(int(sc["max_iters"]), int(sc["res_type"]),
                                    sc["tolerance"])
    if kind == 1:
        return o.compute_source(int(sc["max_iters"]), sc["k_source"],
                                int(sc["res_type"]), sc["tolerance"])
    return o.compute_flux(int(sc["max_iters"]), sc["tolerance"])


def _rel(got, ref, floor=1e-6):
    """Largest error relative to each entry, floored at floor x the peak."""
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.max(np.abs(got - ref) /
                        np.maximum(np.abs(ref), floor * np.abs(ref).max())))


def _peak(got, ref):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.max(np.abs(got - ref)) / np.abs(ref).max())


GOLD = json.load(open(os.path.join(GOLDEN, "reference_results_ls.json")))


@pytest.mark.parametrize("case", sorted(GOLD))
def test_ls_goldens_reproduced_by_reference_fixtures(case):
    """The FP64 OpenMOC build reproduces the committed linear-source
    goldens: iterations, keff to its printed precision, printed fluxes."""
    d = GOLD[case]
    _, sc, arr = load_case(case, "f64")
    assert int(sc["iterations"]) == d["iterations"]
    if "keff" in d:
        assert "%12.5E" % sc["keff"] == "%12.5E" % d["keff"]
    np.testing.assert_allclose(arr["flux"], d["fluxes"], rtol=5e-6)


@pytest.mark.parametrize("case", sorted(GOLD))
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_ls_oracle_matches_reference_goldens(case, precision):
    d = GOLD[case]
    o, _, sc, _ = _oracle(case, precision)
    it = _solve(o, sc)
    assert abs(it - d["iterations"]) <= 1
    if "keff" in d:
        assert abs(o.keff - d["keff"]) < 1.5e-5
    # the goldens were written by a double build; float sweeps of the
    # fixed-source case reach 1.2e-4 on a flux 5e-4 of the peak (OpenMOC's
    # own float build lands on the same values)
    assert _rel(o.phi, d["fluxes"]) < (2e-4 if precision == "f32" else 3e-5)


@pytest.mark.parametrize("case", LS_CASES + LS_CASES_3D)
def test_ls_constants_match_openmoc(case):
    """LinearExpansionGenerator: the 2x2 (3x3 in 3D) inverse per FSR and the
    source constants per FSR and group (G2 by its definition here, by a
    rational accurate to 1e-6 in the reference)."""
    o, p, _, arr = _oracle(case, "f64")
    flat = o.constants()
    assert flat == 0
    assert _peak(o.ilem, arr["ls_ilem"]) < 1e-6
    assert _peak(o.src_const, arr["ls_src_constants"]) < 1e-5


@pytest.mark.parametrize("case", LS_CASES + LS_CASES_3D)
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_ls_oracle_solve_matches_openmoc(case, precision):
    o, p, sc, arr = _oracle(case, precision, threads=2)
    it = _solve(o, sc)
    assert abs(it - int(sc["iterations"])) <= 1
    assert abs(o.keff - sc["keff"]) < 1e-5
    assert _rel(o.phi, arr["flux"]) < 5e-5
    assert _peak(o.mom, arr["ls_moments"]) < 3e-4


@pytest.mark.parametrize("case", LS_PROBE_CASES)
def test_ls_oracle_hooks_match_openmoc(case):
    o, p, sc, arr = _oracle(case, "f32")
    R, G = p.num_fsrs, p.num_groups
    o.constants()
    o.phi[:] = arr["probe_phi_in"]
    o.mom[:] = arr["probe_mom_in"]
    o.phi_old[:] = arr["probe_phi_old"]
    o.keff = sc["probe_keff_in"]
    o.start[:] = arr["probe_start_flux_in"]
    o.compute_sources(100)
    np.testing.assert_allclose(o.reduced, arr["probe_reduced_sources"], rtol=1e-6)
    assert _peak(o.red_xyz, arr["probe_reduced_xyz"]) < 1e-5
    o.sweep()
    ref = arr["probe_phi_sweep"].reshape(R, G)
    got = o.phi.reshape(R, G)
    assert np.max(np.abs(got - ref) / np.abs(ref).max(axis=0)) < 5e-5
    mref = arr["probe_mom_sweep"].reshape(R, 3, G)
    mgot = o.mom.reshape(R, 3, G)
    assert np.max(np.abs(mgot - mref) / np.abs(mref).max(axis=(0, 1))) < 5e-4
    sref = arr["probe_start_flux_out"]
    assert np.max(np.abs(o.start - sref)) <= 2e-4 * np.max(np.abs(sref))
    o.add_source()
    assert _rel(o.phi, arr["probe_phi_addsrc"]) < 2e-5
    assert _peak(o.mom, arr["probe_mom_addsrc"]) < 5e-4
    o.compute_keff()
    assert abs(o.keff - sc["probe_keff_out"]) < 1e-6
    f = o.normalize()
    assert abs(f / sc["probe_norm_factor"] - 1) < 1e-6
    assert _peak(o.mom, arr["probe_mom_norm"]) < 5e-4
    assert abs(o.residual_of(1) - sc["probe_residual_fission"]) < 1e-6


def test_ls_fixture_positions_inside_their_regions():
    """Re-centred start positions: every FSR's length-weighted segment
    midpoints average to ~0 (the centroid), in both precisions' fixtures."""
    for case in LS_CASES:
        p, _, arr = load_case(case, "f64")
        x = arr["ls_seg_x"].astype(np.float64)
        y = arr["ls_seg_y"].astype(np.float64)
        d = arr["ls_ang_dir"].reshape(-1, 2)
        w = arr["ls_ang_wgt"]
        T = p.num_tracks
        a = np.repeat(p.track_ang, np.diff(p.seg_off))
        L = p.seg_len.astype(np.float64)
        mx = x + 0.5 * L * d[a, 0]
        my = y + 0.5 * L * d[a, 1]
        wl = w[a] * L
        sx = np.bincount(p.seg_fsr, wl * mx, p.num_fsrs)
        sy = np.bincount(p.seg_fsr, wl * my, p.num_fsrs)
        vol = np.bincount(p.seg_fsr, wl, p.num_fsrs)
        size = np.sqrt(vol)
        assert np.max(np.abs(sx / vol) / size) < 1e-5, case
        assert np.max(np.abs(sy / vol) / size) < 1e-5, case
        assert T == len(p.seg_off) - 1


def test_ls_3d_fixture_positions_inside_their_regions():
    """The 3D fixture's re-centred start positions: every FSR's
    weight-and-length-weighted segment midpoints average to ~0 in x, y and
    z, and the angle rows hold unit directions."""
    for case in LS_CASES_3D:
        p, _, arr = load_case(case, "f64")
        d = arr["ls_ang_dir"].reshape(-1, 2)
        sth, cth = arr["ls_pol_sin"], arr["ls_pol_cos"]
        assert np.allclose(sth ** 2 + cth ** 2, 1.0)
        a = np.repeat(p.track_ang, np.diff(p.seg_off))
        L = p.seg_len.astype(np.float64)
        w = (arr["ls_ang_wgt"] * arr["ls_pol_wgt"])[a] * L
        vol = np.bincount(p.seg_fsr, w, p.num_fsrs)
        size = np.cbrt(vol)
        for key, u in (("ls_seg_x", d[a, 0] * sth[a]), ("ls_seg_y", d[a, 1] * sth[a]),
                       ("ls_seg_z", cth[a])):
            m = arr[key].astype(np.float64) + 0.5 * L * u
            c = np.bincount(p.seg_fsr, w * m, p.num_fsrs) / vol
            assert np.max(np.abs(c) / size) < 1e-5, (case, key)


def test_ls_oracle_stabilization_identities():
    """The oracle's moment stabilization: GLOBAL with factor 1 (a zero
    stabilizing flux, scaled by 1) and DIAGONAL on a problem without
    negative within-group scattering change nothing; GLOBAL with factor 0.5
    changes the moments."""
    o0 = _oracle("pin7_ls", "f64")[0]
    o0.compute_eigenvalue(6, 1, 1e-30)
    for kind, factor in ((2, 1.0), (0, 1.0)):
        o = _oracle("pin7_ls", "f64")[0]
        o.stabilize_transport(factor, kind)
        o.compute_eigenvalue(6, 1, 1e-30)
        assert o.keff == o0.keff
        np.testing.assert_array_equal(o.mom, o0.mom)
        np.testing.assert_array_equal(o.phi, o0.phi)
    o = _oracle("pin7_ls", "f64")[0]
    o.stabilize_transport(0.5, 2)
    o.compute_eigenvalue(6, 1, 1e-30)
    assert np.abs(o.mom - o0.mom).max() > 0
