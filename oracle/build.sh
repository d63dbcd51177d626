#!/bin/bash
# Builds the C restatement of the CPU solver (oracle/moc_oracle.c) as two
# shared libraries, float and double, into oracle/_build/, and a host-only
# build of the library's pin-lattice track generator
# (openmoc_gb300/csrc/lattice.cpp, no CUDA code) so that the timed CPU
# baseline can lay down its tracks without loading the GPU library.  Test
# infrastructure only: loaded by tests/, the smoke check and bench.py's CPU
# baseline, never by the product library.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/.." && pwd)
OUT=$HERE/_build
mkdir -p "$OUT"
CFLAGS="-O3 -fopenmp -fPIC -shared -std=c11 -Wall -Wno-unknown-pragmas"
gcc $CFLAGS -DORACLE_REAL=float  "$HERE/moc_oracle.c" -lm -o "$OUT/libmoc_oracle_f32.so" &
pids=($!)
gcc $CFLAGS -DORACLE_REAL=double "$HERE/moc_oracle.c" -lm -o "$OUT/libmoc_oracle_f64.so" &
pids+=($!)
# the same flags the library build gives this file: no FMA contraction, so
# the segments are the same as the GPU library's on every host
g++ -O3 -fopenmp -fPIC -shared -std=c++17 -ffp-contract=off -I "$ROOT/include" \
    "$ROOT/openmoc_gb300/csrc/lattice.cpp" -o "$OUT/libmoc_tracks.so" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
