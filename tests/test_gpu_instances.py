"""Instances: K cross-section sets over one track laydown solved together
(moc_set_instances; one sweep per iteration carries every instance's groups,
sources, keff and the normalisation stay per instance).

Each instance against the same problem solved alone on the GPU and against
the FP64 oracle after a fixed number of iterations, on a 2D lattice (7
groups, so group pairs straddle two instances) and on an extruded 3D pin;
converged, against the separate converged solves; and the requests the
context refuses.
"""
import numpy as np
import pytest

from openmoc_gb300 import GB300Solver, instances
from openmoc_gb300 import lattice as lat
from openmoc_gb300._native import MOCError
from oracle.oracle import FISSION_SOURCE, Oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.abs(b)))


def _sets(base, K, G, config):
    """K lognormal(0, 0.05) perturbations of the base problem's materials."""
    xs = []
    for k in range(K):
        mats = lat._fuel_mod(config, G, 1, perturb=(500 + k, 0.05))
        xs.append(lat.pack_materials(mats))
    return xs


def _lattice3(G=7):
    pm = np.zeros((3, 3), np.int32)
    pm[1, 1] = 1
    return lat.lattice(3, 3, pm, lat._fuel_mod(0, G, 1), 1, num_azim=16, spacing=0.1,
                       bc=(lat.REFLECTIVE, lat.VACUUM, lat.REFLECTIVE, lat.VACUUM))


def _pin3d(G=7):
    return lat.lattice(1, 1, np.zeros((1, 1), np.int32), lat._fuel_mod(0, G, 1), 1,
                       num_azim=8, spacing=0.1,
                       extrude=dict(height=2.0, fuel_height=1.6, z_spacing=0.4,
                                    num_polar=4))


def _alone(p, iters, thr=1e-30):
    s = GB300Solver(p)
    s.setConvergenceThreshold(thr)
    s.computeEigenvalue(iters, FISSION_SOURCE)
    out = s.getKeff(), s.getFluxes(), s.getNumIterations()
    s.close()
    return out


@pytest.mark.parametrize("make,K,iters", [(_lattice3, 3, 15), (_pin3d, 4, 10)])
def test_instances_match_separate_solves_and_oracle(make, K, iters):
    base = make()
    G = base.num_groups
    sets = _sets(base, K, G, 0)
    wide = instances(base, sets)
    s = GB300Solver(wide)
    s.setInstances(K)
    s.setConvergenceThreshold(1e-30)
    s.computeEigenvalue(iters, FISSION_SOURCE)
    assert s.getNumIterations() == iters
    keffs = s.getInstanceKeffs()
    fluxes = s.getInstanceFluxes()
    assert fluxes.shape == (K, base.num_fsrs, G)
    s.close()
    for k in range(K):
        p = base.with_xs(*sets[k])
        k_alone, f_alone, _ = _alone(p, iters)
        assert abs(keffs[k] - k_alone) < 2e-6, (k, keffs[k], k_alone)
        assert _rel(fluxes[k], f_alone) < 2e-5, k
        o = Oracle(p, "f64")
        o.compute_eigenvalue(iters, FISSION_SOURCE, 1e-30)
        assert abs(keffs[k] - o.keff) < 2e-6, k
        assert _rel(fluxes[k].ravel(), o.phi) < 2e-5, k


def test_instances_converge_to_the_separate_answers():
    base = _lattice3()
    K = 3
    sets = _sets(base, K, base.num_groups, 0)
    s = GB300Solver(instances(base, sets))
    s.setInstances(K)
    s.setConvergenceThreshold(1e-6)
    s.computeEigenvalue(2000, FISSION_SOURCE)
    keffs = s.getInstanceKeffs()
    fluxes = s.getInstanceFluxes()
    n = s.getNumIterations()
    s.close()
    for k in range(K):
        k_alone, f_alone, n_alone = _alone(base.with_xs(*sets[k]), 2000, 1e-6)
        assert n >= n_alone   # the set stops when its slowest instance does
        assert abs(keffs[k] - k_alone) < 1e-5
        assert _rel(fluxes[k], f_alone) < 1e-4


def test_instances_refuse_what_they_do_not_cover():
    base = _lattice3()
    wide = instances(base, _sets(base, 2, base.num_groups, 0))
    s = GB300Solver(wide)
    with pytest.raises(MOCError, match="multiple"):
        s.setInstances(3)          # 14 groups are not 3 instances
    s.setInstances(2)
    with pytest.raises(MOCError, match="moc_compute_eigenvalue only"):
        s.computeSource(10, 1.0)
    s.close()
