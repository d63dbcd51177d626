"""The benchmarked configurations at full size: the CUDA path against the
FP64 references at a fixed number of source iterations.

* 17 x 17 assembly, 70 groups, 64 azimuthal, 0.05 cm (the configuration the
  throughput is quoted on), with the sweep-kernel instance the benchmark
  runs (8 lanes per track direction x 5 group pairs per lane, hardware ex2
  evaluator) and each source contraction (3xTF32 tensor cores, FP32 CUDA
  cores): 20 iterations against OpenMOC's FP64 CPUSolver on the same tracks
  (tests/golden/openmoc_assembly70_f64.json) and against the FP64 oracle's
  full flux.
* 51 x 51 core, 7 groups, 128 azimuthal, 0.03 cm: 6 iterations against
  OpenMOC FP64 and the FP64 oracle.
* 17 x 17 assembly extruded to 20 cm, 7 groups, explicit 3D tracks (the
  library's extrusion): 4 iterations against the FP64 oracle, stored
  segments and on-the-fly segmentation.

Bar: keff within 1e-5 absolute and FSR scalar fluxes within 1e-4 max
relative (every FSR and group against the oracle; OpenMOC's 4096-flux
sample and per-group sums against OpenMOC).
"""
import numpy as np
import pytest

from conftest import errors_against_golden, load_openmoc_config_golden
from openmoc_gb300 import GB300Solver
from openmoc_gb300 import lattice as lt
from openmoc_gb300.solver import EXP_INTRINSIC, FISSION_SOURCE
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

KEFF_TOL = 1e-5
FLUX_TOL = 1e-4


def max_rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.max(np.abs(a - b) / np.abs(b)))


def gpu_solve(p, iters, shape=None, sources=None, formation=None):
    s = GB300Solver(device=0)
    if formation:
        s.setSegmentFormation(formation)
    s.setTrackGenerator(p)
    s.setConvergenceThreshold(1e-30)
    if shape:
        s.setSweepShape(*shape)
        s.useExponentialIntrinsic()
    if sources:
        s.setSourceContraction(sources)
    s.computeEigenvalue(iters, FISSION_SOURCE)
    info = dict(iterations=s.getNumIterations(), shape=s.getSweepShape(),
                exp=s.getExponential(),
                sources=s.getSourceContraction() if not formation else None)
    k, flux = s.getKeff(), s.getFluxes()
    s.close()
    return k, flux, info


@pytest.fixture(scope="module")
def assembly70():
    g = load_openmoc_config_golden("assembly70")
    p = lt.assembly_17x17()
    o = Oracle(p, "f64")
    o.compute_eigenvalue(int(g["iterations"]), FISSION_SOURCE, 1e-30)
    return p, g, o


@pytest.mark.parametrize("sources", ["tf32x3", "fp32"])
def test_assembly70_headline_instance(assembly70, sources):
    p, g, o = assembly70
    iters = int(g["iterations"])
    k, flux, info = gpu_solve(p, iters, shape=(8, 5), sources=sources)
    assert info["iterations"] == iters
    assert info["shape"] == (8, 5) and info["exp"] == EXP_INTRINSIC
    assert info["sources"] == sources
    dk, df, ds = errors_against_golden(k, flux, g)
    assert dk <= KEFF_TOL, dk
    assert df <= FLUX_TOL, df
    assert ds <= FLUX_TOL, ds
    assert abs(k - o.keff) <= KEFF_TOL
    assert max_rel(flux, o.phi) <= FLUX_TOL


def test_core51():
    g = load_openmoc_config_golden("core51")
    p = lt.core_51x51(device=0)
    iters = int(g["iterations"])
    k, flux, info = gpu_solve(p, iters)
    assert info["iterations"] == iters
    dk, df, ds = errors_against_golden(k, flux, g)
    assert dk <= KEFF_TOL, dk
    assert df <= FLUX_TOL, df
    assert ds <= FLUX_TOL, ds
    o = Oracle(p, "f64")
    o.compute_eigenvalue(iters, FISSION_SOURCE, 1e-30)
    assert abs(k - o.keff) <= KEFF_TOL
    assert max_rel(flux, o.phi) <= FLUX_TOL


def test_assembly3d():
    p = lt.assembly_17x17_3d()
    iters = 4
    o = Oracle(p, "f64")
    o.compute_eigenvalue(iters, FISSION_SOURCE, 1e-30)
    for formation, shape in ((None, (4, 1)), (None, None), ("otf", None)):
        k, flux, info = gpu_solve(p, iters, shape=shape, formation=formation)
        assert info["iterations"] == iters
        assert abs(k - o.keff) <= KEFF_TOL, (formation, shape, k, o.keff)
        assert max_rel(flux, o.phi) <= FLUX_TOL, (formation, shape)
