"""The C oracle (oracle/moc_oracle.c) against OpenMOC itself.

Pins the oracle before it is trusted as the checker of the CUDA path:
  * OpenMOC's own regression goldens (tests/test_forward_pin_cell and
    tests/test_forward_pin_cell_70g results_true.dat, copied into
    tests/golden/reference_results.json) are reproduced by the fixtures
    that OpenMOC's library wrote, and by the oracle;
  * every fixture case: iterations, keff and fluxes of the oracle against
    OpenMOC's CPUSolver (FP_PRECISION=float and =double builds);
  * hook by hook (sources, sweep, add-source, keff, normalisation,
    residuals) from the same converged state.
"""
import json
import os

import numpy as np
import pytest

from conftest import BALANCE_CASES, CASES, CASES_3D, GOLDEN, SRC_CASES, STAB_CASES, load_case
from oracle.oracle import Oracle


def _solve(oracle, sc):
    kind = int(sc["run_kind"])
    if kind == 0:
        return oracle.compute_eigenvalue(int(sc["max_iters"]), int(sc["res_type"]),
                                         sc["tolerance"])
    if kind == 1:
        return oracle.compute_source(int(sc["max_iters"]), sc["k_source"],
                                     int(sc["res_type"]), sc["tolerance"])
    return oracle.compute_flux(int(sc["max_iters"]), sc["tolerance"])


def test_reference_goldens_reproduced_by_reference_fixtures():
    """The FP64 OpenMOC build used for the fixtures reproduces OpenMOC's
    committed goldens: iteration count, keff to its printed precision and
    the printed fluxes."""
    ref = json.load(open(os.path.join(GOLDEN, "reference_results.json")))
    for case, d in ref.items():
        _, sc, arr = load_case(case, "f64")
        assert int(sc["iterations"]) == d["iterations"]
        assert "%12.5E" % sc["keff"] == "%12.5E" % d["keff"]
        np.testing.assert_allclose(arr["flux"], d["fluxes"], rtol=5e-6)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_oracle_matches_reference_goldens(precision):
    ref = json.load(open(os.path.join(GOLDEN, "reference_results.json")))
    for case, d in ref.items():
        p, sc, _ = load_case(case, precision)
        o = Oracle(p, precision, num_threads=1)
        it = _solve(o, sc)
        assert abs(it - d["iterations"]) <= 1
        assert abs(o.keff - d["keff"]) < 1.5e-5
        np.testing.assert_allclose(o.phi, d["fluxes"], rtol=2e-5)


@pytest.mark.parametrize("case", CASES + SRC_CASES + CASES_3D + BALANCE_CASES + STAB_CASES)
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_oracle_solve_matches_openmoc(case, precision):
    """Including keff from the neutron balance and the three transport
    stabilizations."""
    p, sc, arr = load_case(case, precision)
    o = Oracle(p, precision, num_threads=2)
    o.configure(sc)
    it = _solve(o, sc)
    assert abs(it - int(sc["iterations"])) <= 1
    assert abs(o.keff - sc["keff"]) < 1e-5
    np.testing.assert_allclose(o.phi, arr["flux"], rtol=1e-5)


@pytest.mark.parametrize("case", CASES + BALANCE_CASES)
def test_oracle_hooks_match_openmoc(case):
    p, sc, arr = load_case(case, "f32")
    o = Oracle(p, "f32", num_threads=1)
    o.configure(sc)
    o.phi[:] = arr["probe_phi_in"]
    o.phi_old[:] = arr["probe_phi_old"]
    o.keff = sc["probe_keff_in"]
    o.start[:] = arr["probe_start_flux_in"]
    o.compute_sources(100)
    np.testing.assert_allclose(o.reduced, arr["probe_reduced_sources"], rtol=1e-6)
    o.sweep()
    # raw sweep tallies can cancel; compare on the scale of each group
    ref = arr["probe_phi_sweep"].reshape(p.num_fsrs, p.num_groups)
    got = o.phi.reshape(p.num_fsrs, p.num_groups)
    scale = np.abs(ref).max(axis=0)
    assert np.max(np.abs(got - ref) / scale) < 5e-5
    sref = arr["probe_start_flux_out"]
    # OpenMOC's rational exponential is accurate to 2e-6 absolute in F1
    assert np.max(np.abs(o.start - sref)) <= 2e-4 * np.max(np.abs(sref))
    o.add_source()
    np.testing.assert_allclose(o.phi, arr["probe_phi_addsrc"], rtol=1e-5)
    o.compute_keff()
    assert abs(o.keff - sc["probe_keff_out"]) < 1e-6
    f = o.normalize()
    assert abs(f / sc["probe_norm_factor"] - 1) < 1e-6
    assert abs(o.residual_of(1) - sc["probe_residual_fission"]) < 1e-6
    assert abs(o.residual_of(0) - sc["probe_residual_flux"]) < 1e-5
    assert abs(o.residual_of(2) - sc["probe_residual_total"]) < 1e-6


def test_fixture_fsr_ids_identical_across_precisions():
    """FSR numbering, tracks and links are integer data: the FP32 and FP64
    OpenMOC builds must produce them bit-identically."""
    for case in CASES + SRC_CASES + CASES_3D:
        a, _, _ = load_case(case, "f32")
        b, _, _ = load_case(case, "f64")
        for name in ("seg_fsr", "seg_off", "next", "flags", "track_ang", "fsr_mat"):
            np.testing.assert_array_equal(getattr(a, name), getattr(b, name))
        np.testing.assert_array_equal(a.seg_len, b.seg_len)
