"""Host-side validation of packed problems (no GPU)."""
import numpy as np
import pytest

from conftest import load_case


def test_fixture_problem_validates():
    p, _, _ = load_case("lat3_g2_vac")
    p.validate()
    assert p.fluxes_per_track == 2 * 3
    assert p.integrations_per_sweep == 2 * 6 * p.num_segments
    assert p.num_fissionable_fsrs() > 0


@pytest.mark.parametrize("mutate, msg", [
    (lambda p: p.seg_fsr.__setitem__(0, p.num_fsrs), "FSR id"),
    (lambda p: p.seg_fsr.__setitem__(0, -1), "FSR id"),
    (lambda p: p.next.__setitem__(3, p.num_tracks), "next-track"),
    (lambda p: p.seg_len.__setitem__(2, np.nan), "length"),
    (lambda p: p.seg_len.__setitem__(2, -1.0), "negative segment"),
    (lambda p: p.sigma_t.__setitem__(0, 0.0), "sigma_t"),
    (lambda p: p.sigma_s.__setitem__(1, np.inf), "sigma_s"),
    (lambda p: p.fsr_mat.__setitem__(0, 99), "material"),
    (lambda p: p.track_ang.__setitem__(0, p.num_angles), "angle"),
])
def test_validation_rejects(mutate, msg):
    p, _, _ = load_case("lat3_g2_vac")
    mutate(p)
    with pytest.raises(ValueError, match=msg):
        p.validate()


def test_seg_off_must_cover_segments():
    p, _, _ = load_case("pin_c5g7")
    p.seg_off = p.seg_off.copy()
    p.seg_off[-1] -= 1
    with pytest.raises(ValueError):
        p.validate()
