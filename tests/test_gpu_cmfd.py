"""CMFD-accelerated eigenvalue solves on the GPU (GB300Solver.setCmfd)
against OpenMOC's own CMFD-accelerated CPUSolver runs, and against the
unaccelerated GPU solve.

  * the reference fixtures (a reflective 3 x 3 lattice on a 3 x 3 mesh with
    two coarse groups, a 5 x 5 lattice with vacuum on two sides on a 5 x 5
    mesh): iterations within one, keff within 1e-5, fluxes within 1e-4;
  * a generated 17 x 17 assembly: CMFD converges to the unaccelerated
    answer in fewer iterations, with a pin-cell mesh and a coarser one;
  * rejected requests.
"""
import numpy as np
import pytest

from conftest import CMFD_CASES, CMFD_SOR, load_case

pytestmark = pytest.mark.gpu


def _rel(got, ref, floor):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.max(np.abs(got - ref) /
                        np.maximum(np.abs(ref), floor * np.abs(ref).max())))


def _cmfd(p, groups, solver="cells", sor=1.5):
    """solver: "cells" / "block" (the device coarse solve cell-parallel or
    on one block) or "host" (FP64 on the host)."""
    from openmoc_gb300 import Cmfd
    c = Cmfd()
    c.useHostSolver(solver == "host")
    if solver != "host":
        c.setDeviceSolver(solver)
    nx = p.cmfd_geometry["widths_x"].size
    ny = p.cmfd_geometry["widths_y"].size
    c.setLatticeStructure(nx, ny)
    if groups is not None:
        c.setGroupStructure(groups)
    c.setSORRelaxationFactor(sor)
    c.setCMFDRelaxationFactor(0.7)
    if "k_nearest" in p.cmfd_geometry:
        c.setKNearest(int(p.cmfd_geometry["k_nearest"][0]))
    return c


@pytest.mark.parametrize("case", sorted(CMFD_CASES))
@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("solver", ["cells", "block", "host"])
def test_gpu_cmfd_matches_openmoc(case, precision, solver):
    """The coarse solve on the GPU in FP32 (cell-parallel or on one block)
    or on the host in FP64; the linear-source case through GB300LSSolver
    (moments prolonged, no Larsen factor)."""
    from openmoc_gb300 import GB300LSSolver, GB300Solver
    p, sc, arr = load_case(case, precision)
    s = (GB300LSSolver if p.linear_source is not None else GB300Solver)(device=0)
    s.setConvergenceThreshold(sc["tolerance"])
    s.setTrackGenerator(p)
    s.setCmfd(_cmfd(p, CMFD_CASES[case], solver, CMFD_SOR[case]))
    s.computeEigenvalue(int(sc["max_iters"]), int(sc["res_type"]))
    info = s.getCmfdInfo()
    assert info["enabled"] and info["power_iterations"] > 25
    assert abs(s.getNumIterations() - int(sc["iterations"])) <= 1
    assert abs(s.getKeff() - sc["keff"]) < 1e-5
    assert _rel(s.getFluxes(), arr["flux"].reshape(p.num_fsrs, -1), 1e-4) < 1e-4
    s.close()


def _assembly(G=7):
    from openmoc_gb300 import lattice as lat
    return lat.assembly_17x17(num_groups=G, num_azim=16, spacing=0.1)


@pytest.mark.parametrize("mesh", [17, 1])
def test_gpu_cmfd_converges_to_unaccelerated_answer(mesh):
    """A 17 x 17 assembly with vacuum on two sides: the CMFD solve (pin-cell
    mesh, or one coarse cell per 17 x 17 block = no spatial coupling)
    reaches the unaccelerated solution; the pin-cell mesh in far fewer
    iterations."""
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    mats = lat._fuel_mod(1, 7, 1)
    pm = np.zeros((17, 17), np.int32)
    for (r, c) in lat.GUIDE_TUBES_17x17:
        pm[r, c] = 1
    p = lat.lattice(17, 17, pm, mats, 1, num_azim=16, spacing=0.1,
                    bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM))
    # an FP32 coarse solve leaves a residual floor near 2e-7
    tol = 1e-6
    ref = GB300Solver(p, device=0)
    ref.setConvergenceThreshold(tol)
    ref.computeEigenvalue(3000, 1)
    n_plain = ref.getNumIterations()
    s = GB300Solver(device=0)
    s.setConvergenceThreshold(tol)
    s.setTrackGenerator(p)
    c = Cmfd()
    c.setLatticeStructure(mesh, mesh)
    c.setGroupStructure([[1, 2, 3], [4, 5, 6, 7]])
    s.setCmfd(c)
    s.computeEigenvalue(3000, 1)
    n_cmfd = s.getNumIterations()
    assert abs(s.getKeff() - ref.getKeff()) < 5e-6
    assert _rel(s.getFluxes(), ref.getFluxes(), 1e-3) < 1e-4
    if mesh == 17:
        assert n_cmfd < 0.5 * n_plain, (n_cmfd, n_plain)
    info = s.getCmfdInfo()
    assert info["power_iterations"] > 25 and info["linear_iterations"] > 25
    old, new = s.getCmfdFluxes()
    assert old.shape == (mesh * mesh, 2) and np.isfinite(new).all()
    ref.close()
    s.close()


def test_gpu_cmfd_detach_restores_plain_solve():
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    p = lat.square_lattice(3, 7, 16, 0.1, 0, water_pins=[(1, 1)])
    a = GB300Solver(p, device=0)
    a.computeEigenvalue(1000, 1)
    b = GB300Solver(p, device=0)
    c = Cmfd()
    c.setLatticeStructure(3, 3)
    b.setCmfd(c)
    b.computeEigenvalue(1000, 1)
    assert b.getNumIterations() < a.getNumIterations()
    b.setCmfd(None)
    b.computeEigenvalue(1000, 1)
    assert b.getNumIterations() == a.getNumIterations()
    assert not b.getCmfdInfo()["enabled"]
    a.close()
    b.close()


def test_gpu_cmfd_bad_requests_raise():
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300._native import MOCError
    p = lat.square_lattice(3, 7, 16, 0.1, 0)
    s = GB300Solver(p, device=0)
    c = Cmfd()
    c.setLatticeStructure(2, 2)          # mesh lines cut the pins
    with pytest.raises(MOCError):
        s.setCmfd(c)
    c = Cmfd()
    c.setLatticeStructure(3, 3)
    c.setGroupStructure([[1, 2], [3]])   # does not cover 7 groups
    with pytest.raises(MOCError):
        s.setCmfd(c)
    s.close()


def test_gpu_cmfd_uses_native_library():
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    p = lat.square_lattice(3, 7, 16, 0.1, 0)
    s = GB300Solver(p, device=0)
    c = Cmfd()
    c.setLatticeStructure(3, 3)
    s.setCmfd(c)
    n0 = s.getLaunchCount()
    s.computeEigenvalue(3, 1)
    assert s.getLaunchCount() >= n0 + 3 * 6
    s.close()


@pytest.mark.parametrize("solver,k", [("cells", 0), ("block", 0), ("host", 0),
                                      ("cells", 3), ("block", 3)])
def test_gpu_cmfd_matches_oracle_step_by_step(solver, k):
    """A generated 5 x 5 lattice (vacuum on +x and +y, water pins) on a pin
    mesh with two coarse groups, a fixed number of iterations: keff, fluxes
    and the coarse fluxes of the last coarse solve against the FP64 oracle
    CMFD (oracle/cmfd_oracle.py)."""
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    from oracle.cmfd_oracle import CmfdOracle, cmfd_eigenvalue
    from oracle.oracle import Oracle
    mats = lat._fuel_mod(2, 7, 1)
    pm = np.zeros((5, 5), np.int32)
    for (r, c) in [(1, 1), (2, 3), (3, 2)]:
        pm[r, c] = 1
    p = lat.lattice(5, 5, pm, mats, 1, num_azim=16, spacing=0.1,
                    bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM))
    groups = [[1, 2, 3], [4, 5, 6, 7]]
    c = Cmfd()
    c.setLatticeStructure(5, 5)
    c.setGroupStructure(groups)
    c.useHostSolver(solver == "host")
    if solver != "host":
        c.setDeviceSolver(solver)
    if k:
        c.setKNearest(k)
    mesh, keep = c.mesh(p)
    g = p.cmfd_geometry
    cm = CmfdOracle(p, 5, 5, keep[0], keep[1], keep[2], g["end_face"], g["bc"],
                    keep[4], g["edc_mu"], g["edc_w"], k_nearest=k,
                    centroid=g["fsr_centroid"], origin=(g["bounds"][0], g["bounds"][2]))
    o = Oracle(p, "f64", num_threads=8)
    iters = 8
    cmfd_eigenvalue(o, cm, iters, 1, 1e-30)
    s = GB300Solver(device=0)
    s.setConvergenceThreshold(1e-30)
    s.setTrackGenerator(p)
    s.setCmfd(c)
    s.computeEigenvalue(iters, 1)
    assert s.getNumIterations() == iters
    assert abs(s.getKeff() - o.keff) < 2e-6
    R = p.num_fsrs
    assert _rel(s.getFluxes(), o.phi.reshape(R, -1), 1e-4) < 2e-5
    old, new = s.getCmfdFluxes()
    assert np.max(np.abs(new - cm.new_flux)) < 1e-4 * np.abs(cm.new_flux).max()
    assert np.max(np.abs(old - cm.old_flux)) < 1e-4 * np.abs(cm.old_flux).max()
    assert abs(s.getCmfdInfo()["keff"] - cm.keff) < 2e-6
    s.close()


def test_gpu_cmfd_linear_source_converges_to_unaccelerated_answer():
    """A generated 5 x 5 lattice with the linear source, vacuum on +x and
    +y: CMFD (moments prolonged) reaches the unaccelerated linear-source
    solution in fewer iterations."""
    from openmoc_gb300 import Cmfd, GB300LSSolver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    mats = lat._fuel_mod(2, 7, 1)
    pm = np.zeros((5, 5), np.int32)
    for (r, c) in [(1, 1), (2, 3), (3, 2)]:
        pm[r, c] = 1
    p = lat.lattice(5, 5, pm, mats, 1, num_azim=16, spacing=0.1,
                    bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM),
                    linear_source=True)
    ref = GB300LSSolver(p, device=0)
    ref.setConvergenceThreshold(1e-6)
    ref.computeEigenvalue(3000, 1)
    s = GB300LSSolver(p, device=0)
    s.setConvergenceThreshold(1e-6)
    c = Cmfd()
    c.setLatticeStructure(5, 5)
    c.setGroupStructure([[1, 2, 3], [4, 5, 6, 7]])
    c.setSORRelaxationFactor(1.0)
    s.setCmfd(c)
    s.computeEigenvalue(3000, 1)
    assert s.getNumIterations() < ref.getNumIterations()
    assert abs(s.getKeff() - ref.getKeff()) < 5e-6
    assert _rel(s.getFluxes(), ref.getFluxes(), 1e-3) < 1e-4
    R, G = p.num_fsrs, p.num_groups
    m, mr = s.getFluxMoments(), ref.getFluxMoments()
    assert np.max(np.abs(m - mr)) < 2e-4 * np.abs(mr).max()
    ref.close()
    s.close()


def test_gpu_cmfd_generic_instance_converges_to_unaccelerated_answer():
    """More than 8 coarse groups take the generic instance of the device
    coarse solve (512 threads, a cell's groups looped at run time): a
    16-group assembly with every group its own coarse group reaches the
    unaccelerated answer in fewer iterations."""
    from openmoc_gb300 import Cmfd, GB300Solver
    p = _assembly(16)
    tol = 1e-6
    ref = GB300Solver(p, device=0)
    ref.setConvergenceThreshold(tol)
    ref.computeEigenvalue(20000, 1)
    n_plain = ref.getNumIterations()
    assert n_plain < 20000
    s = GB300Solver(p, device=0)
    s.setConvergenceThreshold(tol)
    c = Cmfd()
    c.setLatticeStructure(17, 17)
    s.setCmfd(c)
    s.computeEigenvalue(20000, 1)
    info = s.getCmfdInfo()
    assert info["enabled"] and not info["failed"]
    assert s.getNumIterations() < n_plain, (s.getNumIterations(), n_plain)
    assert abs(s.getKeff() - ref.getKeff()) < 5e-6
    assert _rel(s.getFluxes(), ref.getFluxes(), 1e-3) < 1e-4
    ref.close()
    s.close()


def test_gpu_cmfd_cell_parallel_refuses_more_than_eight_coarse_groups():
    """The cell-parallel coarse solve keeps a cell's row in registers for up
    to 8 coarse groups: asked for it with 16, the solve is refused; "auto"
    takes the one-block solve instead."""
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300._native import MOCError
    p = _assembly(16)
    for kind in ("cells", "auto"):
        s = GB300Solver(p, device=0)
        c = Cmfd()
        c.setLatticeStructure(17, 17)
        c.setDeviceSolver(kind)
        s.setCmfd(c)
        if kind == "cells":
            with pytest.raises(MOCError, match="cell-parallel"):
                s.computeEigenvalue(3, 1)
        else:
            s.computeEigenvalue(3, 1)
            assert s.getCmfdInfo()["power_iterations"] > 0
        s.close()


def test_gpu_cmfd_core_mesh_matches_oracle_step_by_step():
    """The regime of the 51 x 51 core's CMFD benchmark: a 51 x 51 pin mesh
    (2,601 cells, 1,300 and 1,301 of each red-black colour: the one-block
    device solve updates two cells of a colour in a thread, the
    cell-parallel one spreads the cells over a cluster of four blocks that
    exchange their border cells) with two coarse groups, three fuel sets in
    a checkerboard of assemblies, vacuum on +x and +y.  A fixed number of iterations (a coarser quadrature than
    the benchmark's keeps the oracle quick): keff, fluxes, the coarse fluxes
    and the coarse keff of the last coarse solve against the FP64 oracle
    CMFD (oracle/cmfd_oracle.py)."""
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    from oracle.cmfd_oracle import CmfdOracle, cmfd_eigenvalue
    from oracle.oracle import Oracle
    mats = lat._fuel_mod(3, 7, 3)
    pm = np.zeros((51, 51), np.int32)
    for ar in range(3):
        for ac in range(3):
            block = np.full((17, 17), (ar + ac) % 3, np.int32)
            for (r, c) in lat.GUIDE_TUBES_17x17:
                block[r, c] = 3
            pm[17 * ar:17 * ar + 17, 17 * ac:17 * ac + 17] = block
    p = lat.lattice(51, 51, pm, mats, 3, num_azim=8, spacing=0.1,
                    bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM))
    groups = [[1, 2, 3], [4, 5, 6, 7]]
    c = Cmfd()
    c.setLatticeStructure(51, 51)
    c.setGroupStructure(groups)
    mesh, keep = c.mesh(p)
    g = p.cmfd_geometry
    cm = CmfdOracle(p, 51, 51, keep[0], keep[1], keep[2], g["end_face"], g["bc"],
                    keep[4], g["edc_mu"], g["edc_w"], centroid=g["fsr_centroid"],
                    origin=(g["bounds"][0], g["bounds"][2]))
    o = Oracle(p, "f64")
    iters = 6
    cmfd_eigenvalue(o, cm, iters, 1, 1e-30)
    R = p.num_fsrs
    # the FP32 device coarse solve (cell-parallel, one block) and the FP64
    # host one
    for solver in ("cells", "block", "host"):
        c.useHostSolver(solver == "host")
        if solver != "host":
            c.setDeviceSolver(solver)
        s = GB300Solver(device=0)
        s.setConvergenceThreshold(1e-30)
        s.setTrackGenerator(p)
        s.setCmfd(c)
        s.computeEigenvalue(iters, 1)
        info = s.getCmfdInfo()
        assert s.getNumIterations() == iters
        assert info["enabled"] and not info["failed"]
        assert abs(s.getKeff() - o.keff) < 2e-6, solver
        assert _rel(s.getFluxes(), o.phi.reshape(R, -1), 1e-4) < 2e-5, solver
        old, new = s.getCmfdFluxes()
        assert old.shape == (51 * 51, 2)
        assert np.max(np.abs(new - cm.new_flux)) < 1e-4 * np.abs(cm.new_flux).max(), solver
        assert np.max(np.abs(old - cm.old_flux)) < 1e-4 * np.abs(cm.old_flux).max(), solver
        assert abs(info["keff"] - cm.keff) < 2e-6, solver
        s.close()


@pytest.mark.parametrize("kind,factor", [("GLOBAL", 0.5), ("YAMAMOTO", 0.5)])
def test_gpu_cmfd_with_stabilization_matches_oracle(kind, factor):
    """Transport stabilization inside the CMFD loop (stabilizeFlux after the
    CMFD update, before the normalisation, src/Solver.cpp:1616-1640): the
    5 x 5 lattice of the step-by-step test, 8 iterations, against the FP64
    oracle CMFD with the oracle's stabilization hooks."""
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    from oracle.cmfd_oracle import CmfdOracle, cmfd_eigenvalue
    from oracle.oracle import Oracle
    mats = lat._fuel_mod(2, 7, 1)
    pm = np.zeros((5, 5), np.int32)
    for (r, c) in [(1, 1), (2, 3), (3, 2)]:
        pm[r, c] = 1
    p = lat.lattice(5, 5, pm, mats, 1, num_azim=16, spacing=0.1,
                    bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM))
    c = Cmfd()
    c.setLatticeStructure(5, 5)
    c.setGroupStructure([[1, 2, 3], [4, 5, 6, 7]])
    mesh, keep = c.mesh(p)
    g = p.cmfd_geometry
    cm = CmfdOracle(p, 5, 5, keep[0], keep[1], keep[2], g["end_face"], g["bc"],
                    keep[4], g["edc_mu"], g["edc_w"], k_nearest=0,
                    centroid=g["fsr_centroid"], origin=(g["bounds"][0], g["bounds"][2]))
    o = Oracle(p, "f64", num_threads=8)
    o.stabilize_transport(factor, {"YAMAMOTO": 1, "GLOBAL": 2}[kind])
    iters = 8
    cmfd_eigenvalue(o, cm, iters, 1, 1e-30)
    s = GB300Solver(device=0)
    s.setConvergenceThreshold(1e-30)
    s.setTrackGenerator(p)
    s.setCmfd(c)
    s.stabilizeTransport(factor, kind)
    s.computeEigenvalue(iters, 1)
    assert s.getNumIterations() == iters
    assert abs(s.getKeff() - o.keff) < 2e-6
    R = p.num_fsrs
    assert _rel(s.getFluxes(), o.phi.reshape(R, -1), 1e-4) < 2e-5
    s.close()
