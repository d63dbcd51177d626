"""The library's pin-lattice track generator (csrc/lattice.cpp) against the
tracks OpenMOC's TrackGenerator produced for the fixtures: integer data
(FSR ids, segment offsets, links, flags, angles, materials) bit-identical,
segment lengths bit-identical in float, FSR volumes to float accumulation
order, and the benchmark-size counts OpenMOC reports."""
import numpy as np
import pytest

from conftest import load_case
from openmoc_gb300 import lattice as lt

CASES = {
    "pin7_synth": lambda: lt.pin_cell(7, 32, 0.05, config=0),
    "lat3_g2_vac": lambda: lt.lattice(
        3, 3, np.array([[0, 0, 0], [0, 1, 0], [0, 0, 0]]), lt._fuel_mod(2, 2), 1,
        num_azim=16, spacing=0.1, bc=(lt.REFLECTIVE, lt.VACUUM, lt.REFLECTIVE, lt.VACUUM)),
    "lat2_g16": lambda: lt.square_lattice(2, 16, 8, 0.1, 3, [(1, 1)]),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_generator_matches_openmoc_tracks(case):
    ref, _, _ = load_case(case, "f32")
    p = CASES[case]()
    for k in ("num_fsrs", "num_tracks", "num_segments", "num_angles", "num_polar_half"):
        assert getattr(p, k) == getattr(ref, k), k
    for k in ("seg_off", "seg_fsr", "next", "flags", "track_ang", "fsr_mat"):
        np.testing.assert_array_equal(getattr(p, k), getattr(ref, k), err_msg=k)
    for k in ("seg_len", "weights", "inv_sin", "sigma_t", "sigma_s", "nu_sigma_f", "chi"):
        np.testing.assert_array_equal(getattr(p, k), getattr(ref, k), err_msg=k)
    np.testing.assert_allclose(p.fsr_vol, ref.fsr_vol, rtol=1e-6)


def test_benchmark_sizes_match_openmoc_counts():
    p = lt.assembly_17x17()
    assert (p.num_fsrs, p.num_tracks, p.num_segments) == (9248, 17500, 1971864)
    assert p.num_groups == 70 and p.num_polar_half == 3
    p.validate()


def test_generator_rejects_bad_specs():
    with pytest.raises(RuntimeError, match="num_azim"):
        lt.pin_cell(7, 30, 0.05)
    with pytest.raises(RuntimeError, match="num_polar"):
        lt.lattice(1, 1, np.zeros((1, 1)), lt._fuel_mod(0, 2), 1, num_azim=8,
                   spacing=0.1, num_polar=5)
