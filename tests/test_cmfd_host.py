"""CMFD host side without a GPU: the settings object, the mesh laid over a
generated lattice, and the lattice's CMFD geometry against what OpenMOC
records for the same lattice (tests/golden/cmfd_lat3, made by
make_fixtures.cpp with Geometry::setCmfd)."""
import numpy as np
import pytest

from conftest import CMFD_CASES, load_case


def _lat3():
    from openmoc_gb300 import lattice as lat
    return lat.square_lattice(3, 7, 16, 0.1, 0, water_pins=[(1, 1)])


def test_cmfd_settings_validate():
    from openmoc_gb300 import Cmfd
    from openmoc_gb300._native import MOCError
    c = Cmfd()
    with pytest.raises(MOCError):
        c.setGroupStructure([[1, 2], [4]])          # not contiguous
    with pytest.raises(MOCError):
        c.setGroupStructure([[2, 3]])               # does not start at 1
    with pytest.raises(MOCError):
        c.setSORRelaxationFactor(2.0)
    with pytest.raises(MOCError):
        c.setCMFDRelaxationFactor(0.0)
    with pytest.raises(MOCError):
        c.setKNearest(10)
    with pytest.raises(MOCError):
        c.setLatticeStructure(3, 3, 2)
    c.setKNearest(1)
    c.setGroupStructure([[1, 2, 3], [4, 5, 6, 7]])
    assert c.getNumCmfdGroups() == 2


def test_cmfd_mesh_over_generated_lattice():
    from openmoc_gb300 import Cmfd
    from openmoc_gb300._native import MOCError
    p = _lat3()
    c = Cmfd()
    c.setLatticeStructure(3, 3)
    m, keep = c.mesh(p)
    cell = keep[2]
    assert m.num_x == 3 and m.num_y == 3 and m.num_cmfd_groups == 7
    assert np.bincount(cell, minlength=9).tolist() == [32] * 9
    # every FSR's lattice-cell box lies in its coarse cell, y from y-min
    box = p.cmfd_geometry["fsr_box"]
    assert np.all(np.floor((box[:, 2] + 1e-9 + 1.89) / 1.26) == cell // 3)
    assert np.all(np.floor((box[:, 0] + 1e-9 + 1.89) / 1.26) == cell % 3)
    c.setLatticeStructure(1, 1)
    m, keep = c.mesh(p)
    assert (keep[2] == 0).all()
    c.setLatticeStructure(2, 2)
    with pytest.raises(MOCError):
        c.mesh(p)
    c = Cmfd()
    c.setWidths([[1.26, 2.52], [2.52, 1.26]])
    m, keep = c.mesh(p)
    assert np.bincount(keep[2], minlength=4).tolist() == [64, 128, 32, 64]


def test_cmfd_lattice_geometry_matches_openmoc():
    """The generated 3 x 3 lattice is the fixture's geometry: the same
    Larsen-EDC quadrature, the same numbers of track ends on each face and
    of FSRs in each coarse cell."""
    p = _lat3()
    q, sc, arr = load_case("cmfd_lat3", "f64")
    g, r = p.cmfd_geometry, q.cmfd_geometry
    np.testing.assert_allclose(g["edc_mu"], r["edc_mu"], rtol=1e-12)
    np.testing.assert_allclose(g["edc_w"], r["edc_w"], rtol=1e-12)
    np.testing.assert_allclose(g["bounds"], r["bounds"], atol=1e-12)
    assert g["bc"].tolist() == r["bc"].tolist() == [1, 1, 1, 1]
    assert np.bincount(g["end_face"] + 1, minlength=5).tolist() == \
        np.bincount(r["end_face"] + 1, minlength=5).tolist()
    assert np.bincount(r["fsr_cell"], minlength=9).tolist() == [32] * 9
    assert q.num_tracks == p.num_tracks and q.num_fsrs == p.num_fsrs


@pytest.mark.parametrize("case", sorted(CMFD_CASES))
def test_cmfd_fixtures_hold_a_mesh(case):
    from openmoc_gb300 import Cmfd
    p, sc, _ = load_case(case, "f32")
    g = p.cmfd_geometry
    assert (p.linear_source is not None) == case.endswith("_ls")
    assert g["end_face"].size == 2 * p.num_tracks
    assert g["fsr_cell"].size == p.num_fsrs
    c = Cmfd()
    c.setLatticeStructure(g["widths_x"].size, g["widths_y"].size)
    if CMFD_CASES[case] is not None:
        c.setGroupStructure(CMFD_CASES[case])
    m, keep = c.mesh(p)
    assert np.array_equal(keep[2], g["fsr_cell"])
    assert m.num_edc_angles == g["edc_mu"].size


def test_cmfd_lattice_centroids_match_openmoc():
    """The generated lattice's FSR centroids (the k-nearest update's input)
    against OpenMOC's Geometry::getFSRCentroid for the same lattice, FSR by
    FSR after matching FSRs by centroid (the two number FSRs differently)."""
    p = _lat3()
    q, sc, arr = load_case("cmfd_lat3_k3", "f64")
    g = p.cmfd_geometry["fsr_centroid"].reshape(-1, 2)
    r = q.cmfd_geometry["fsr_centroid"].reshape(-1, 2)
    assert g.shape == r.shape
    d = np.sqrt(((g[:, None, :] - r[None, :, :]) ** 2).sum(-1))
    nearest = d.argmin(1)
    assert np.unique(nearest).size == g.shape[0]      # one to one
    assert d.min(1).max() < 2e-6
