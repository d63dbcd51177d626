"""The library's pin-lattice track generator (csrc/lattice.cpp) against the
tracks OpenMOC's TrackGenerator produced for the fixtures: integer data
(FSR ids, segment offsets, links, flags, angles, materials) bit-identical,
segment lengths bit-identical in float, FSR volumes to float accumulation
order, and the benchmark-size counts OpenMOC reports."""
import os

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


def _extruded_pin(dz=0.4, polar=4, azim=4, spacing=0.1):
    from openmoc_gb300 import lattice
    mats = [lattice.synthetic_xs(lattice.SEED + 5, 7, True),
            lattice.synthetic_xs(lattice.SEED + 1005, 7, False)]
    return lattice.lattice(1, 1, np.zeros((1, 1), np.int32), mats, 1, num_azim=azim,
                           spacing=spacing, fuel_rings=2, fuel_sectors=4, mod_sectors=4,
                           extrude=dict(height=2.0, fuel_height=1.6, z_spacing=dz,
                                        num_polar=polar))


def test_extrusion_volumes_links_and_regions():
    """The axial extrusion: the same FSRs as OpenMOC's explicit-3D fixture
    (radial FSRs below the fuel top, one moderator region above), volumes
    that sum to the zones' exact volumes, and links that pair up: a flux
    passed on at one end of a track comes back, along the reverse path, to
    that same end."""
    p = _extruded_pin()
    ref, _, _ = load_case("pin3d_g7")
    assert p.solve_3d == 1 and p.num_polar_half == 1
    assert p.num_fsrs == ref.num_fsrs == 13
    area = 1.26 * 1.26
    assert p.fsr_vol[:-1].sum() == pytest.approx(area * 1.6, rel=1e-6)
    assert p.fsr_vol[-1] == pytest.approx(area * 0.4, rel=1e-6)
    # the top region has the moderator's material, as in OpenMOC's fixture
    assert p.fsr_mat[-1] == 1
    assert np.all(p.inv_sin == 1.0)
    T = p.num_tracks
    nxt = p.next.reshape(T, 2)
    for t in range(T):
        f = p.flags[t]
        if f & 4:     # forward end: into n forward (bit 0) or backward
            n = nxt[t, 0]
            if f & 1:
                assert nxt[n, 1] == t and p.flags[n] & 8 and not p.flags[n] & 2
            else:
                assert nxt[n, 0] == t and p.flags[n] & 4 and not p.flags[n] & 1
        if f & 8:     # backward end: into n forward (bit 1) or backward
            n = nxt[t, 1]
            if f & 2:
                assert nxt[n, 1] == t and p.flags[n] & 8 and p.flags[n] & 2
            else:
                assert nxt[n, 0] == t and p.flags[n] & 4 and p.flags[n] & 1
    # every line starts and ends on the vacuum bottom / top
    assert np.count_nonzero((p.flags & 4) == 0) == np.count_nonzero((p.flags & 8) == 0)


def test_extrusion_is_openmocs_3d_laydown():
    """The extruded pin with OpenMOC's fixture parameters (4 azimuthal, 4
    polar, 0.1 cm radial, 0.4 cm axial) is OpenMOC's own explicit-3D
    laydown (TrackGenerator3D, in the fixture pin3d_g7): the same tracks in
    the same order, segment by segment the same regions (up to the FSR
    numbering) and lengths, the same angle rows and weights, and the same
    connections wherever the flux is passed on."""
    p = _extruded_pin()
    ref, _, _ = load_case("pin3d_g7")
    assert (p.num_tracks, p.num_segments) == (ref.num_tracks, ref.num_segments)
    assert np.array_equal(p.seg_off, ref.seg_off)
    assert np.array_equal(p.track_ang, ref.track_ang)
    assert np.allclose(p.weights, ref.weights, rtol=1e-6, atol=0)
    assert np.allclose(p.seg_len, ref.seg_len, rtol=1e-6, atol=0)
    # one FSR of ours for each of OpenMOC's, everywhere
    pairs = set(zip(p.seg_fsr.tolist(), ref.seg_fsr.tolist()))
    assert len(pairs) == len({a for a, _ in pairs}) == len({b for _, b in pairs}) == 13
    for a, b in pairs:
        assert p.fsr_vol[a] == pytest.approx(ref.fsr_vol[b], rel=1e-5)
    f, g = ref.flags, p.flags
    assert np.array_equal(f & 12, g & 12)
    fwd, bwd = (f & 4) != 0, (f & 8) != 0
    nr, nm = ref.next.reshape(-1, 2), p.next.reshape(-1, 2)
    assert np.array_equal(nr[fwd, 0], nm[fwd, 0]) and np.array_equal(f[fwd] & 1, g[fwd] & 1)
    assert np.array_equal(nr[bwd, 1], nm[bwd, 1]) and np.array_equal(f[bwd] & 2, g[bwd] & 2)


def test_extrusion_ls_geometry_is_openmocs():
    """The linear-source geometry of the extruded pin (moc_lattice_export_ls3d)
    against OpenMOC's own (pin3d_ls: CPULSSolver on TrackGenerator3D's
    laydown of the same pin): angle rows, weights, sin / cos theta exactly;
    segment starts relative to the centroids to a float rounding; 3D
    centroids to 1e-7."""
    from openmoc_gb300 import lattice
    mats = [lattice.synthetic_xs(lattice.SEED + 5, 7, True),
            lattice.synthetic_xs(lattice.SEED + 1005, 7, False)]
    p = lattice.lattice(1, 1, np.zeros((1, 1), np.int32), mats, 1, num_azim=4,
                        spacing=0.1, fuel_rings=2, fuel_sectors=4, mod_sectors=4,
                        extrude=dict(height=2.0, fuel_height=1.6, z_spacing=0.4,
                                     num_polar=4), linear_source=True)
    ref, _, arr = load_case("pin3d_ls", "f64")
    ls = p.linear_source
    assert np.array_equal(p.seg_off, ref.seg_off)
    for k in ("ang_dir", "ang_wgt", "pol_sin", "pol_cos"):
        assert np.array_equal(ls[k], arr["ls_" + k]), k
    assert np.allclose(ls["pol_wgt"], arr["ls_pol_wgt"], rtol=1e-14, atol=0)
    for k in ("seg_x", "seg_y", "seg_z"):
        assert np.max(np.abs(ls[k].astype(np.float64) - arr["ls_" + k])) < 2e-7, k
    pairs = dict(zip(p.seg_fsr.tolist(), ref.seg_fsr.tolist()))
    c, cr = ls["centroid"].reshape(-1, 3), arr["ls_centroid"].reshape(-1, 3)
    assert max(np.abs(c[a] - cr[b]).max() for a, b in pairs.items()) < 1e-7
    # each 3D track runs along its row's direction
    d = p.track_ends[:, 3:] - p.track_ends[:, :3]
    d /= np.linalg.norm(d, axis=1)[:, None]
    a = p.track_ang
    u = np.stack([ls["ang_dir"][2 * a] * ls["pol_sin"][a],
                  ls["ang_dir"][2 * a + 1] * ls["pol_sin"][a], ls["pol_cos"][a]], 1)
    assert np.abs(d - u).max() < 1e-12


def test_assembly3d_is_openmocs_3d_laydown():
    """The 3D benchmark assembly (17 x 17 extruded to 20 cm, 16 azimuthal,
    6 polar, 0.1 / 0.5 cm) against OpenMOC's own laydown of it
    (tests/golden/openmoc_assembly3d_laydown.json, written by
    make_laydown3d_golden.py from TrackGenerator3D): the track and segment
    counts, checksums of the segment counts, angle rows, transfer flags and
    connections in track order, and the lengths, weights and volumes."""
    from conftest import GOLDEN, track_checksum
    from openmoc_gb300 import lattice
    import json
    with open(os.path.join(GOLDEN, "openmoc_assembly3d_laydown.json")) as fh:
        g = json.load(fh)
    p = lattice.assembly_17x17_3d()
    assert (p.num_fsrs, p.num_tracks, p.num_segments) == (
        g["num_fsrs"], g["num_tracks"], g["num_segments"])
    nseg = np.diff(p.seg_off).astype(np.int32)
    flags, nxt = p.flags, p.next.reshape(-1, 2)
    fwd, bwd = (flags & 4) != 0, (flags & 8) != 0
    masked = (flags & 12) | np.where(fwd, flags & 1, 0) | np.where(bwd, flags & 2, 0)
    c = g["checksums"]
    assert track_checksum(nseg) == int(c["nseg"])
    assert track_checksum(p.track_ang.astype(np.int32)) == int(c["row"])
    assert track_checksum(masked.astype(np.uint8)) == int(c["flags"])
    assert track_checksum(np.where(fwd, nxt[:, 0], -1).astype(np.int64)) == int(c["next_fwd"])
    assert track_checksum(np.where(bwd, nxt[:, 1], -1).astype(np.int64)) == int(c["next_bwd"])
    lsum = np.add.reduceat(p.seg_len.astype(np.float64), p.seg_off[:-1])
    rows = np.bincount(p.track_ang, weights=lsum, minlength=len(g["row_length"]))
    assert np.allclose(rows, g["row_length"], rtol=1e-6, atol=0)
    above = p.seg_len[p.seg_fsr == p.num_fsrs - 1].astype(np.float64).sum()
    assert above == pytest.approx(g["length_above_fuel"], rel=1e-6)
    assert np.allclose(p.weights, g["weights"], rtol=1e-6, atol=0)
    vol = np.sort(p.fsr_vol.astype(np.float64))
    assert np.allclose(np.quantile(vol, np.linspace(0, 1, 101)), g["volume_quantiles"],
                       rtol=1e-5, atol=0)
    assert vol.sum() == pytest.approx(g["volume_total"], rel=1e-6)


def test_extrusion_keff_is_openmocs():
    """On OpenMOC's own laydown the FP64 oracle gives the keff of OpenMOC's
    explicit-3D run (fixture pin3d_g7, stopped by the same 1e-5 criterion)
    within the parity bar."""
    from oracle.oracle import Oracle
    _, sc, _ = load_case("pin3d_g7", "f64")
    o = Oracle(_extruded_pin(), "f64", num_threads=2)
    o.compute_eigenvalue(int(sc["max_iters"]), int(sc["res_type"]), sc["tolerance"])
    assert abs(o.keff - sc["keff"]) < 1e-5


def _otf_pieces(p):
    """The pieces the on-the-fly sweep cuts for every 3D track, in traversal
    order (a restatement of otf_sweep.cu's cut() in double precision),
    merged like the explicit generator merges consecutive pieces of one
    region."""
    o = p.otf
    trk = o["trk"].reshape(-1, 4)
    tf = o["trk_f"].reshape(-1, 4).astype(np.float64)
    ang = o["ang"].reshape(-1, 4).astype(np.float64)
    above = int(o["above_fsr"][0])
    out = []
    for t in range(p.num_tracks):
        t2, first, n, rev = (int(v) for v in trk[t])
        a0, span, w0 = tf[t, 0], tf[t, 1], tf[t, 2]
        cot, icot, isin = ang[p.track_ang[t], :3]
        rb = int(o["rad_off"][t2])
        total = float(o["rad_total"][t2])
        pieces = []
        for k in range(n):
            idx = first - k if rev else first + k
            l = float(o["rad_len"][rb + idx])
            c0 = float(o["rad_start"][rb + idx])
            s = (total - c0 - l) - a0 if rev else c0 - a0
            us, ue = max(s, 0.0), min(s + l, span)
            if not ue > us:
                continue
            ws, we = w0 + us * cot, w0 + ue * cot
            below = int(o["rad_fsr"][rb + idx])
            if max(ws, we) <= 0 or min(ws, we) >= 0:
                pieces.append((below if max(ws, we) <= 0 else above, (ue - us) * isin))
            else:
                uc = us - ws * icot
                a_, b_ = (below, above) if ws < 0 else (above, below)
                pieces.append((a_, (uc - us) * isin))
                pieces.append((b_, (ue - uc) * isin))
        merged = []
        for f, l in pieces:
            if l <= 1e-10:
                continue
            if merged and merged[-1][0] == f:
                merged[-1][1] += l
            else:
                merged.append([f, l])
        out.append(merged)
    return out


def test_otf_description_reproduces_explicit_segments():
    """The on-the-fly track description of an extruded lattice cuts the same
    3D segments as the explicit generator stores (FSR ids exactly, lengths to
    float rounding)."""
    mats = lt._fuel_mod(4, 7, 1)
    pm = np.zeros((2, 2), np.int32)
    pm[0, 1] = 1
    p = lt.lattice(2, 2, pm, mats, 1, num_azim=8, spacing=0.1,
                        extrude=dict(height=2.0, fuel_height=1.6, z_spacing=0.4,
                                     num_polar=4))
    pieces = _otf_pieces(p)
    for t in range(p.num_tracks):
        b, e = p.seg_off[t], p.seg_off[t + 1]
        got = pieces[t]
        assert [f for f, _ in got] == list(p.seg_fsr[b:e]), t
        np.testing.assert_allclose([l for _, l in got], p.seg_len[b:e], rtol=2e-5,
                                   atol=2e-6)
