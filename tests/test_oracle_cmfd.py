"""The CMFD restatement of the oracle (oracle/cmfd_oracle.py over the C
transport oracle's current-tallying sweep) against OpenMOC's own
CMFD-accelerated solves (tests/golden/cmfd_*, Geometry::setCmfd in
make_fixtures.cpp): the same iteration count, keff within 1e-6, fluxes
within 1e-5."""
import numpy as np
import pytest

from conftest import CMFD_CASES, load_case
from oracle.cmfd_oracle import CmfdOracle, cmfd_eigenvalue
from oracle.oracle import Oracle


def cmfd_oracle_for(p, groups, **kw):
    g = p.cmfd_geometry
    go = None
    if groups is not None:
        go = np.concatenate([[e] * len(gr) for e, gr in enumerate(groups)])
    if "k_nearest" in g:
        kw.setdefault("k_nearest", int(g["k_nearest"][0]))
        kw.setdefault("centroid", g["fsr_centroid"])
        kw.setdefault("origin", (g["bounds"][0], g["bounds"][2]))
    return CmfdOracle(p, g["widths_x"].size, g["widths_y"].size, g["widths_x"],
                      g["widths_y"], g["fsr_cell"], g["end_face"], g["bc"], go,
                      g["edc_mu"], g["edc_w"], **kw)


@pytest.mark.parametrize("case,precision", [("cmfd_lat3", "f64"),
                                            ("cmfd_lat3", "f32"),
                                            ("cmfd_lat5_vac", "f64"),
                                            ("cmfd_lat3_k3", "f64")])
def test_cmfd_oracle_matches_openmoc(case, precision):
    p, sc, arr = load_case(case, precision)
    cm = cmfd_oracle_for(p, CMFD_CASES[case])
    o = Oracle(p, precision, num_threads=8)
    it = cmfd_eigenvalue(o, cm, int(sc["max_iters"]), int(sc["res_type"]),
                         sc["tolerance"])
    assert it == int(sc["iterations"])
    assert abs(o.keff - sc["keff"]) < 1e-6
    f = arr["flux"].reshape(p.num_fsrs, -1).astype(np.float64)
    assert np.max(np.abs(o.phi.reshape(f.shape) - f)) < 1e-5 * np.abs(f).max()
    assert cm.power_iterations > 25


def test_cmfd_oracle_accelerates():
    """The reflective 3 x 3 lattice: fewer iterations than the plain
    source iteration of the oracle, same answer within the tolerance."""
    p, sc, _ = load_case("cmfd_lat3", "f64")
    plain = Oracle(p, "f64", num_threads=8)
    n_plain = plain.compute_eigenvalue(1000, 1, 1e-5)
    assert int(sc["iterations"]) < 0.7 * n_plain
    assert abs(plain.keff - sc["keff"]) < 5e-5
