"""Writes tests/golden/openmoc_assembly3d_laydown.json: a summary of OpenMOC's
own 3D laydown of the extruded 17 x 17 assembly (TrackGenerator3D, 16
azimuthal, 6 polar, 0.1 cm radial, 0.5 cm axial spacing, explicit 3D
segments), from oracle/openmoc_run.cpp's laydown3d mode, which the laydown
of openmoc_gb300.lattice.assembly_17x17_3d is checked against
(tests/test_lattice.py).

Integer data as the order-sensitive checksums of conftest.track_checksum in
track UID order: segment counts, angle rows (a * num_polar + p), the
transfer bits of the flags, and the connecting tracks and direction bits
where the flux is transferred (a vacuum end's link is not used, and its value
is the generator's own); float data as per-row sums of track lengths, the
length above the fuel, the row weights and quantiles of the FSR volumes.

Needs the OpenMOC source tree; run from the repository root:
    REF=<OpenMOC source tree> python tests/golden/make_laydown3d_golden.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
from conftest import track_checksum  # noqa: E402

P = 6


def summarise(d):
    meta = json.load(open(os.path.join(d, "meta.json")))

    def ld(n):
        return np.fromfile(os.path.join(d, n + ".bin"), dtype=meta[n][0])

    flags = ld("flags")
    nxt = ld("next").reshape(-1, 2)
    fwd, bwd = (flags & 4) != 0, (flags & 8) != 0
    masked = (flags & 12) | np.where(fwd, flags & 1, 0) | np.where(bwd, flags & 2, 0)
    rows = (ld("azim") * P + ld("polar")).astype(np.int32)
    lsum = ld("len_sum")
    vol = np.sort(ld("fsr_vol"))
    nrows = int(rows.max()) + 1
    return {
        "config": "17x17 assembly extruded to 20 cm, fuel below 16 cm; "
                  "TrackGenerator3D(16 azimuthal, 6 polar, 0.1 cm, 0.5 cm), EXPLICIT_3D",
        "num_fsrs": int(vol.size),
        "num_tracks": int(flags.size),
        "num_segments": int(ld("nseg").sum()),
        "checksums": {
            "nseg": str(track_checksum(ld("nseg").astype(np.int32))),
            "row": str(track_checksum(rows)),
            "flags": str(track_checksum(masked.astype(np.uint8))),
            "next_fwd": str(track_checksum(np.where(fwd, nxt[:, 0], -1).astype(np.int64))),
            "next_bwd": str(track_checksum(np.where(bwd, nxt[:, 1], -1).astype(np.int64))),
        },
        "row_length": np.bincount(rows, weights=lsum, minlength=nrows).tolist(),
        "length_above_fuel": float(ld("len_top").sum()),
        "weights": ld("weight").tolist(),
        "volume_quantiles": [float(v) for v in np.quantile(vol, np.linspace(0, 1, 101))],
        "volume_total": float(vol.sum()),
    }


def main():
    ref = os.environ.get("REF")
    if not ref:
        sys.exit("REF must name an OpenMOC source tree")
    out = os.path.join(ROOT, "oracle", "_ref")
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"),
                           f"REF={ref}", f"OUT={out}", f"-j{os.cpu_count() or 4}",
                           os.path.join(out, "openmoc_run_f64")])
    with tempfile.TemporaryDirectory() as d:
        subprocess.check_call([os.path.join(out, "openmoc_run_f64"), "assembly3d",
                               "laydown3d", d, str(os.cpu_count() or 4)])
        summary = summarise(d)
    with open(os.path.join(HERE, "openmoc_assembly3d_laydown.json"), "w") as f:
        json.dump(summary, f, indent=1)
    print(summary["num_tracks"], summary["num_segments"])


if __name__ == "__main__":
    main()
