"""The device ray tracer (moc_lattice_generate_device) against the host
generator and OpenMOC.

The host generator reproduces OpenMOC's segments bit for bit on the fixture
geometries (test_lattice.py); the device ray tracer must give the same
segment lengths, FSR ids (first-touch numbering), offsets, links and flags
bit for bit, and the same FSR volumes up to the order of the FP64 sums.
"""
import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu

EXACT = ("seg_len", "seg_fsr", "seg_off", "track_ang", "next", "flags",
         "weights", "inv_sin", "fsr_mat")


def _same(a, b):
    assert (a.num_fsrs, a.num_tracks, a.num_segments) == \
        (b.num_fsrs, b.num_tracks, b.num_segments)
    for k in EXACT:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)
    np.testing.assert_allclose(a.fsr_vol, b.fsr_vol, rtol=2e-7)


@pytest.mark.parametrize("build", [
    lambda dev: __import__("openmoc_gb300.lattice", fromlist=["x"]).pin_cell(7, device=dev),
    lambda dev: __import__("openmoc_gb300.lattice", fromlist=["x"]).square_lattice(
        3, 2, 16, 0.1, 2, [(1, 1)], device=dev),
    lambda dev: __import__("openmoc_gb300.lattice", fromlist=["x"]).assembly_17x17(
        7, device=dev),
], ids=["pin", "3x3", "17x17"])
def test_device_ray_tracing_matches_host(build):
    _same(build(0), build(None))


def test_device_ray_tracing_matches_openmoc_pin_cell():
    from openmoc_gb300 import lattice as lat
    p = lat.pin_cell(7, device=0)
    q, _, _ = load_case("pin7_synth", "f64")
    for k in ("seg_len", "seg_fsr", "seg_off", "track_ang", "next", "flags"):
        np.testing.assert_array_equal(getattr(p, k), getattr(q, k), err_msg=k)
    np.testing.assert_allclose(p.fsr_vol, q.fsr_vol, rtol=5e-7)


def test_device_ray_tracing_large_core_matches_host():
    """51 x 51 pins, 128 azimuthal, 0.03 cm: 59 M segments."""
    from openmoc_gb300 import lattice as lat
    _same(lat.core_51x51(device=0), lat.core_51x51())


def test_device_ray_tracing_vacuum_and_sectors():
    from openmoc_gb300 import lattice as lat
    mats = lat._fuel_mod(5, 4, 2)
    pm = np.array([[0, 1, 2], [2, 0, 1], [1, 2, 0]], np.int32)
    kw = dict(num_azim=12, spacing=0.07, fuel_rings=4, fuel_sectors=4,
              mod_sectors=16, bc=(lat.VACUUM, lat.REFLECTIVE, lat.VACUUM,
                                  lat.REFLECTIVE))
    _same(lat.lattice(3, 3, pm, mats, 2, device=0, **kw),
          lat.lattice(3, 3, pm, mats, 2, **kw))
