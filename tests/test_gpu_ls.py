"""The linear-source CUDA path (GB300LSSolver) against OpenMOC's CPULSSolver
and the linear-source oracle.

  * the expansion constants computed on the GPU against OpenMOC's
    LinearExpansionGenerator output in every linear-source fixture;
  * whole solves (eigenvalue, computeSource, computeFlux with fixed source
    moments and negative fluxes allowed) against OpenMOC FP32 and FP64:
    iterations, keff within 1e-5, scalar fluxes within 1e-4, flux moments;
  * OpenMOC's own linear-source goldens (test_2d_gradient_linear_source,
    test_fixed_linear_source);
  * hook by hook from OpenMOC's converged state;
  * generated lattices against the oracle at fixed iteration counts, for
    every sweep shape (lanes per track direction x group pairs per lane);
  * explicit 3D tracks (x, y and z moments, six expansion coefficients):
    OpenMOC's 3D CPULSSolver fixture, its constants and its solve for every
    sweep shape, and the FP64 oracle at a fixed iteration count.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, LS_CASES, LS_CASES_3D, LS_PROBE_CASES, load_case, ls_arrays
from oracle.oracle import LSOracle

pytestmark = pytest.mark.gpu


def _xyz(xy, R, G):
    """[R][2][G] moments -> [R][3][G] (z = 0)."""
    m = np.zeros((R, 3, G), np.float32)
    m[:, :2, :] = np.asarray(xy, np.float32).reshape(R, 2, G)
    return m


def _solver(case, precision="f32"):
    from openmoc_gb300 import GB300LSSolver
    p, sc, arr = load_case(case, precision)
    s = GB300LSSolver(device=0)
    if sc.get("allow_negative", 0):
        s.allowNegativeFluxes(True)
    s.setConvergenceThreshold(sc["tolerance"])
    s.setTrackGenerator(p)
    if "fixed_source_xy" in arr:
        s.setFixedSourceMoments(_xyz(arr["fixed_source_xy"], p.num_fsrs,
                                     p.num_groups))
    return s, p, sc, arr


def _solve(s, sc):
    kind = int(sc["run_kind"])
    if kind == 0:
        s.computeEigenvalue(int(sc["max_iters"]), int(sc["res_type"]))
    elif kind == 1:
        s.computeSource(int(sc["max_iters"]), sc["k_source"], int(sc["res_type"]))
    else:
        s.computeFlux(int(sc["max_iters"]))


def _rel(got, ref, floor):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.max(np.abs(got - ref) /
                        np.maximum(np.abs(ref), floor * np.abs(ref).max())))


def _peak(got, ref):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.max(np.abs(got - ref)) / np.abs(ref).max())


@pytest.mark.parametrize("case", LS_CASES)
def test_gpu_ls_constants_match_openmoc(case):
    s, p, _, arr = _solver(case, "f64")
    assert s.getNumFlatSourceRegions() == 0
    il, cst = s.getLinearExpansion()
    R, G = p.num_fsrs, p.num_groups
    # FP64 sums on the device, stored in FP32; G2 from its definition here,
    # from a rational accurate to 1e-6 in the reference
    assert _peak(il, arr["ls_ilem"].reshape(R, 3)) < 2e-6
    assert _peak(cst, arr["ls_src_constants"].reshape(R, 3, G)) < 1e-5
    s.close()


@pytest.mark.parametrize("case", LS_CASES)
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_gpu_ls_solve_matches_openmoc(case, precision):
    s, p, sc, arr = _solver(case, precision)
    _solve(s, sc)
    assert abs(s.getNumIterations() - int(sc["iterations"])) <= 1
    assert abs(s.getKeff() - sc["keff"]) < 1e-5
    # parity bar: 1e-4 on every flux above 1e-4 of the peak
    assert _rel(s.getFluxes(), arr["flux"].reshape(p.num_fsrs, -1), 1e-4) < 1e-4
    R, G = p.num_fsrs, p.num_groups
    assert _peak(s.getFluxMoments(), arr["ls_moments"].reshape(R, 3, G)) < 5e-4
    s.close()


GOLD = json.load(open(os.path.join(GOLDEN, "reference_results_ls.json")))


@pytest.mark.parametrize("case", sorted(GOLD))
def test_gpu_ls_reference_goldens(case):
    """OpenMOC's test_2d_gradient_linear_source / test_fixed_linear_source
    results_true.dat, printed to 6 digits from a double build."""
    d = GOLD[case]
    s, p, sc, _ = _solver(case, "f32")
    _solve(s, sc)
    assert abs(s.getNumIterations() - d["iterations"]) <= 1
    if "keff" in d:
        assert abs(s.getKeff() - d["keff"]) < 1.5e-5
    assert _rel(s.getFluxes().ravel(), d["fluxes"], 1e-4) < 2e-4
    s.close()


@pytest.mark.parametrize("case", LS_PROBE_CASES)
def test_gpu_ls_hooks_match_openmoc(case):
    s, p, sc, arr = _solver(case, "f32")
    R, G = p.num_fsrs, p.num_groups
    s.setFluxes(arr["probe_phi_in"])
    s.setOldFluxes(arr["probe_phi_old"])
    s.setFluxMoments(arr["probe_mom_in"].reshape(R, 3, G))
    s.setKeff(sc["probe_keff_in"])
    s.setStartFlux(arr["probe_start_flux_in"])
    s.computeFSRSources(100)
    ref = arr["probe_reduced_sources"].reshape(R, G)
    np.testing.assert_allclose(s.getReducedSources(), ref, rtol=2e-6)
    assert _peak(s.getSourceMoments(), arr["probe_reduced_xyz"].reshape(R, 3, G)) < 1e-5
    s.transportSweep()
    ref = arr["probe_phi_sweep"].reshape(R, G)
    got = s.getFluxes()
    assert np.max(np.abs(got - ref) / np.abs(ref).max(axis=0)) < 5e-5
    mref = arr["probe_mom_sweep"].reshape(R, 3, G)
    mgot = s.getFluxMoments()
    assert np.max(np.abs(mgot - mref) / np.abs(mref).max(axis=(0, 1))) < 5e-4
    sref = arr["probe_start_flux_out"]
    assert np.max(np.abs(s.getStartFlux() - sref)) <= 2e-4 * np.max(np.abs(sref))
    s.addSourceToScalarFlux()
    assert _rel(s.getFluxes(), arr["probe_phi_addsrc"].reshape(R, G), 1e-6) < 3e-5
    assert _peak(s.getFluxMoments(), arr["probe_mom_addsrc"].reshape(R, 3, G)) < 5e-4
    s.computeKeff()
    assert abs(s.getKeff() - sc["probe_keff_out"]) < 1e-6
    f = s.normalizeFluxes()
    assert abs(f / sc["probe_norm_factor"] - 1) < 1e-6
    assert _peak(s.getFluxMoments(), arr["probe_mom_norm"].reshape(R, 3, G)) < 5e-4
    assert abs(s.computeResidual(1) - sc["probe_residual_fission"]) < 1e-6
    s.close()


def _lattice_ls(n, G, num_azim=16, spacing=0.1, bc=None):
    from openmoc_gb300 import lattice as lat
    water = [(n // 2, n // 2)] if n > 1 else []
    mats = lat._fuel_mod(7, G, 1)
    pm = np.zeros((n, n), np.int32)
    for (r, c) in water:
        pm[r, c] = 1
    kw = {} if bc is None else dict(bc=bc)
    return lat.lattice(n, n, pm, mats, 1, num_azim=num_azim, spacing=spacing,
                       linear_source=True, **kw)


@pytest.mark.parametrize("G,shapes", [
    (7, [(1, 4), (2, 2), (4, 1), (8, 1)]),
    (16, [(2, 4), (4, 2), (8, 1), (16, 1)]),
    (70, [(8, 5), (16, 3), (32, 2)]),
])
def test_gpu_ls_lattice_matches_oracle_every_shape(G, shapes):
    """Generated 3 x 3 lattices (vacuum on +x, +y) against the FP64 oracle
    after a fixed number of eigenvalue iterations, for each sweep shape."""
    from openmoc_gb300 import GB300LSSolver
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    p = _lattice_ls(3, G, bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM))
    iters = 12
    o = LSOracle(p, p.linear_source, "f64", num_threads=8)
    o.compute_eigenvalue(iters, 1, 1e-30)
    R = p.num_fsrs
    ref_m = o.mom.reshape(R, 3, G)
    for lps, pairs in shapes:
        s = GB300LSSolver(device=0)
        s.setSweepShape(lps, pairs)
        s.setConvergenceThreshold(1e-30)
        s.setTrackGenerator(p)
        s.computeEigenvalue(iters, 1)
        assert s.getNumIterations() == iters
        assert abs(s.getKeff() - o.keff) < 2e-6, (lps, pairs)
        assert _rel(s.getFluxes(), o.phi.reshape(R, G), 1e-4) < 2e-5, (lps, pairs)
        assert _peak(s.getFluxMoments(), ref_m) < 1e-4, (lps, pairs)
        s.close()


def test_gpu_ls_generated_pin_matches_openmoc_fixture():
    """The lattice generator's linear-source geometry of the synthetic pin
    cell solves to OpenMOC's pin7_ls result."""
    from openmoc_gb300 import GB300LSSolver
    from openmoc_gb300 import lattice as lat
    p = lat.pin_cell(7, linear_source=True)
    _, sc, arr = load_case("pin7_ls", "f64")
    s = GB300LSSolver(p, device=0)
    s.computeEigenvalue(1000, 1)
    assert abs(s.getNumIterations() - int(sc["iterations"])) <= 1
    assert abs(s.getKeff() - sc["keff"]) < 1e-5
    assert _rel(s.getFluxes(), arr["flux"].reshape(p.num_fsrs, -1), 1e-4) < 1e-4
    s.close()


def test_gpu_ls_bad_requests_raise():
    from openmoc_gb300 import GB300LSSolver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300._native import MOCError
    p = lat.pin_cell(7)          # no linear-source geometry
    with pytest.raises(MOCError):
        GB300LSSolver(p, device=0)
    p = lat.pin_cell(7, linear_source=True)
    bad = dict(p.linear_source)
    bad["ang_dir"] = 2.0 * bad["ang_dir"]     # not unit vectors
    with pytest.raises(MOCError):
        GB300LSSolver(p, linear_source=bad, device=0)
    bad = dict(p.linear_source)
    bad["seg_x"] = bad["seg_x"].copy()
    bad["seg_x"][3] = np.nan
    with pytest.raises(MOCError):
        GB300LSSolver(p, linear_source=bad, device=0)
    s = GB300LSSolver(p, device=0)
    with pytest.raises(MOCError):
        s.setSweepShape(1, 6)                 # more pairs than the instances
    with pytest.raises(MOCError):
        s.setFixedSourceMomentByFSR(p.num_fsrs, 1, 0.1, 0.1)
    s.close()


def test_gpu_ls_uses_native_library():
    from openmoc_gb300 import GB300LSSolver
    from openmoc_gb300 import lattice as lat
    p = lat.pin_cell(7, linear_source=True)
    s = GB300LSSolver(p, device=0)
    n0 = s.getLaunchCount()
    s.computeEigenvalue(3, 1)
    assert s.getLaunchCount() > n0 + 3 * 4
    s.close()


@pytest.mark.parametrize("case", LS_CASES_3D)
def test_gpu_ls_3d_constants_match_openmoc(case):
    s, p, _, arr = _solver(case, "f64")
    assert s.getNumFlatSourceRegions() == 0
    il, cst = s.getLinearExpansion()
    R, G = p.num_fsrs, p.num_groups
    assert il.shape == (R, 6) and cst.shape == (R, 6, G)
    assert _peak(il, arr["ls_ilem"].reshape(R, 6)) < 2e-6
    assert _peak(cst, arr["ls_src_constants"].reshape(R, 6, G)) < 1e-5
    s.close()


@pytest.mark.parametrize("case", LS_CASES_3D)
@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("shape", [None, (1, 4), (2, 2), (4, 1), (8, 1)])
def test_gpu_ls_3d_solve_matches_openmoc(case, precision, shape):
    """CPULSSolver on explicit 3D tracks through the 3D linear-source sweep
    (autotuned, then every shape for 7 groups) against OpenMOC FP32 / FP64:
    iterations, keff 1e-5, fluxes 1e-4, x / y / z moments 5e-4 of the
    peak."""
    s, p, sc, arr = _solver(case, precision)
    if shape:
        s.setSweepShape(*shape)
    _solve(s, sc)
    assert abs(s.getNumIterations() - int(sc["iterations"])) <= 1
    assert abs(s.getKeff() - sc["keff"]) < 1e-5
    R, G = p.num_fsrs, p.num_groups
    assert _rel(s.getFluxes(), arr["flux"].reshape(R, G), 1e-4) < 1e-4
    mom = s.getFluxMoments()
    ref = arr["ls_moments"].reshape(R, 3, G)
    assert _peak(mom, ref) < 5e-4
    assert np.abs(mom[:, 2, :]).max() > 0.1 * np.abs(ref[:, 2, :]).max()
    s.close()


def test_gpu_ls_3d_matches_oracle_at_fixed_iterations():
    """The 3D fixture's problem for 10 eigenvalue iterations against the
    FP64 oracle (no convergence test in between): keff, fluxes and the
    three moments."""
    from openmoc_gb300 import GB300LSSolver
    p, _, arr = load_case("pin3d_ls", "f32")
    iters = 10
    o = LSOracle(p, ls_arrays(arr), "f64", num_threads=8)
    o.compute_eigenvalue(iters, 1, 1e-30)
    s = GB300LSSolver(p, device=0)
    s.setConvergenceThreshold(1e-30)
    s.computeEigenvalue(iters, 1)
    R, G = p.num_fsrs, p.num_groups
    assert s.getNumIterations() == iters
    assert abs(s.getKeff() - o.keff) < 2e-6
    assert _rel(s.getFluxes(), o.phi.reshape(R, G), 1e-4) < 2e-5
    assert _peak(s.getFluxMoments(), o.mom.reshape(R, 3, G)) < 1e-4
    s.close()


@pytest.mark.parametrize("G,shapes", [
    (7, [(1, 4), (2, 2), (4, 1), (8, 1)]),
    (16, [(2, 4), (4, 2), (8, 1), (16, 1)]),
])
def test_gpu_ls_3d_lattice_matches_oracle_every_shape(G, shapes):
    """A 2 x 2 lattice extruded into explicit 3D tracks with the generator's
    3D linear-source geometry (moc_lattice_export_ls3d), vacuum at bottom and
    top, against the FP64 oracle after 8 eigenvalue iterations, for each
    sweep shape."""
    from openmoc_gb300 import GB300LSSolver
    from openmoc_gb300 import lattice as lat
    mats = lat._fuel_mod(4, G, 1)
    pm = np.zeros((2, 2), np.int32)
    pm[1, 1] = 1
    p = lat.lattice(2, 2, pm, mats, 1, num_azim=8, spacing=0.1,
                    extrude=dict(height=4.0, fuel_height=3.2, z_spacing=0.4,
                                 num_polar=4), linear_source=True)
    iters = 8
    o = LSOracle(p, p.linear_source, "f64", num_threads=8)
    o.compute_eigenvalue(iters, 1, 1e-30)
    R = p.num_fsrs
    ref_m = o.mom.reshape(R, 3, G)
    for lps, pairs in shapes:
        s = GB300LSSolver(device=0)
        s.setSweepShape(lps, pairs)
        s.setConvergenceThreshold(1e-30)
        s.setTrackGenerator(p)
        s.computeEigenvalue(iters, 1)
        assert s.getNumIterations() == iters
        assert abs(s.getKeff() - o.keff) < 2e-6, (lps, pairs)
        assert _rel(s.getFluxes(), o.phi.reshape(R, G), 1e-4) < 2e-5, (lps, pairs)
        assert _peak(s.getFluxMoments(), ref_m) < 1e-4, (lps, pairs)
        s.close()


def _negative_in_group_scattering(p):
    """p with the water's within-group scattering made negative (as the
    transport-stabilization fixtures' moderator has it)."""
    M, G = p.num_materials, p.num_groups
    ss = np.array(p.sigma_s, np.float32).reshape(M, G, G)
    for g in range(G):
        ss[M - 1, g, g] = -0.05 * abs(ss[M - 1, g, g])
    p.sigma_s = ss.ravel()
    return p


@pytest.mark.parametrize("kind,factor", [("DIAGONAL", 1.0), ("YAMAMOTO", 0.5),
                                         ("GLOBAL", 0.5)])
def test_gpu_ls_stabilization_matches_oracle(kind, factor):
    """Transport stabilization of a linear-source solve (the flat flux and
    the flux moments, CPULSSolver::computeStabilizingFlux / stabilizeFlux)
    against the FP64 oracle after 12 eigenvalue iterations; the moments
    differ from the unstabilized solve's except under YAMAMOTO, whose
    moment branch in the reference leaves them as they are."""
    from openmoc_gb300 import GB300LSSolver
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    G, iters = 7, 12
    p = _negative_in_group_scattering(
        _lattice_ls(3, G, bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM)))
    o = LSOracle(p, p.linear_source, "f64", num_threads=8)
    o.stabilize_transport(factor, {"DIAGONAL": 0, "YAMAMOTO": 1, "GLOBAL": 2}[kind])
    o.compute_eigenvalue(iters, 1, 1e-30)
    s = GB300LSSolver(p, device=0)
    s.stabilizeTransport(factor, kind)
    s.setConvergenceThreshold(1e-30)
    s.computeEigenvalue(iters, 1)
    R = p.num_fsrs
    assert s.getNumIterations() == iters
    assert abs(s.getKeff() - o.keff) < 2e-6
    assert _rel(s.getFluxes(), o.phi.reshape(R, G), 1e-4) < 2e-5
    assert _peak(s.getFluxMoments(), o.mom.reshape(R, 3, G)) < 1e-4
    s.close()


def test_gpu_ls_3d_stabilization_matches_oracle():
    """GLOBAL stabilization on the 3D fixture's problem (x, y and z
    moments) against the FP64 oracle after 10 eigenvalue iterations."""
    from openmoc_gb300 import GB300LSSolver
    p, _, arr = load_case("pin3d_ls", "f32")
    iters = 10
    o = LSOracle(p, ls_arrays(arr), "f64", num_threads=8)
    o.stabilize_transport(0.5, 2)
    o.compute_eigenvalue(iters, 1, 1e-30)
    s = GB300LSSolver(p, device=0)
    s.stabilizeTransport(0.5, "GLOBAL")
    s.setConvergenceThreshold(1e-30)
    s.computeEigenvalue(iters, 1)
    R, G = p.num_fsrs, p.num_groups
    assert abs(s.getKeff() - o.keff) < 2e-6
    assert _rel(s.getFluxes(), o.phi.reshape(R, G), 1e-4) < 2e-5
    assert _peak(s.getFluxMoments(), o.mom.reshape(R, 3, G)) < 1e-4
    s.close()
