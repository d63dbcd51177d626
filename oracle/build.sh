#!/bin/bash
# Builds the C restatement of the CPU solver (oracle/moc_oracle.c) as two
# shared libraries, float and double, into oracle/_build/.  Test
# infrastructure only: loaded by tests/, the smoke check and bench.py's CPU
# baseline, never by the product library.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_build
mkdir -p "$OUT"
CFLAGS="-O3 -fopenmp -fPIC -shared -std=c11 -Wall -Wno-unknown-pragmas"
gcc $CFLAGS -DORACLE_REAL=float  "$HERE/moc_oracle.c" -lm -o "$OUT/libmoc_oracle_f32.so" &
gcc $CFLAGS -DORACLE_REAL=double "$HERE/moc_oracle.c" -lm -o "$OUT/libmoc_oracle_f64.so" &
wait
