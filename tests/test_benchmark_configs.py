"""The benchmark configurations at full size against OpenMOC itself (CPU).

tests/golden/openmoc_<config>_f64.json hold what OpenMOC's FP64 CPUSolver
gives on the pin cell (20 source iterations), the 17 x 17 / 70-group
assembly (20) and the 51 x 51 / 7-group core (6), built through OpenMOC's
Geometry / Lattice / TrackGenerator (oracle/openmoc_run.cpp).

* The library's track generator reproduces OpenMOC's tracks on each of them:
  integer data bit for bit (checksums of FSR ids, offsets, angles, links,
  flags and materials); segment lengths and FSR volumes to one unit in the
  last place, checked through exact sums of the values rounded to a 2^-24 cm
  (lengths) and 2^-20 cm^2 (volumes) grid, plain and index-weighted.  A
  length below 2 cm that rounds k units in the last place apart moves the
  plain sum by at most 2k grid steps; the bound is 2 grid steps per 100,000
  values (16 at least).  Measured: on the 17 x 17 assembly 5 of the
  1,971,864 float lengths (segments of 2e-4 cm) and 160 of the 9,248
  volumes differ by one unit in the last place; on the 51 x 51 core 6,617
  of the 59,097,984 lengths differ by 1 to 7 units (all below 0.27 cm; net
  39 grid steps, 2.3e-6 cm in all) and 804 of the 83,232 volumes by one.
  So the GPU solves of these configurations run on OpenMOC's own inputs.
* The FP64 oracle (oracle/moc_oracle.c) matches OpenMOC FP64 there after
  the same iterations: keff to 1e-6 and fluxes to 1e-5, inside the
  1e-5 / 1e-4 parity bar the GPU is held to (the oracle evaluates
  (1 - exp(-x)) / x exactly, OpenMOC with its rational approximation).
"""
import pytest

from conftest import (errors_against_golden, load_openmoc_config_golden, quantised_sums,
                      track_checksum, wrapped_difference)
from openmoc_gb300 import lattice as lt

BUILDERS = {
    "pin7": lambda: lt.pin_cell(7, 32, 0.05, config=0),
    "assembly70": lambda: lt.assembly_17x17(),
    "core51": lambda: lt.core_51x51(),
}


@pytest.mark.parametrize("config", sorted(BUILDERS))
def test_tracks_are_openmoc_tracks(config):
    g = load_openmoc_config_golden(config)
    p = BUILDERS[config]()
    assert (p.num_fsrs, p.num_tracks, p.num_segments, p.num_groups) == (
        g["num_fsrs"], g["num_tracks"], g["num_segments"], g["num_groups"])
    for k, v in g["checksums"].items():
        assert track_checksum(getattr(p, k)) == int(v), k
    for k, bits, n in (("seg_len", 24, p.num_segments), ("fsr_vol", 20, p.num_fsrs)):
        ref = g[f"{k}_q{bits}"]
        got = quantised_sums(getattr(p, k), bits)
        bound = max(16, 2 * n // 100_000)
        assert abs(wrapped_difference(got[0], ref[0])) <= bound, k
        assert abs(wrapped_difference(got[1], ref[1])) <= 1009 * bound, k


@pytest.mark.parametrize("config", ["pin7", "assembly70"])
def test_fp64_oracle_matches_openmoc_fp64(config):
    from oracle.oracle import FISSION_SOURCE, Oracle
    g = load_openmoc_config_golden(config)
    p = BUILDERS[config]()
    o = Oracle(p, "f64")
    o.compute_eigenvalue(int(g["iterations"]), FISSION_SOURCE, 1e-30)
    dk, df, ds = errors_against_golden(o.keff, o.phi, g)
    assert dk < 1e-6, dk
    assert df < 1e-5, df
    assert ds < 1e-5, ds
