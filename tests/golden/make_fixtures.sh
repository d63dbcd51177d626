#!/bin/bash
# Regenerates the golden fixtures in tests/golden/ from OpenMOC's own C++
# library, built from the reference sources by oracle/ref.mk.  Needs the
# reference tree (REF=<OpenMOC source tree>); run from the repo root:
#   bash tests/golden/make_fixtures.sh [case]
set -euo pipefail
: "${REF:?REF must name an OpenMOC source tree}"
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
OUT=$ROOT/oracle/_ref
make -s -f "$ROOT/oracle/ref.mk" REF="$REF" OUT="$OUT" -j"$(nproc)"
CXXF="-O2 -fopenmp -std=c++11 -w -DGCC -DOPENMP -DVEC_ALIGNMENT=64 -I$REF/src"
g++ $CXXF -DFP_PRECISION=float -DSINGLE -DVEC_LENGTH=8 \
    -DCMFD_PRECISION=float -DLINALG_TOL=1E-7 \
    "$HERE/make_fixtures.cpp" "$OUT/libopenmoc_f32.a" -o "$OUT/make_fixtures_f32"
g++ $CXXF -DFP_PRECISION=double -DVEC_LENGTH=4 \
    -DCMFD_PRECISION=double -DLINALG_TOL=1E-15 \
    "$HERE/make_fixtures.cpp" "$OUT/libopenmoc_f64.a" -o "$OUT/make_fixtures_f64"
"$OUT/make_fixtures_f32" "$HERE" "${1:-}"
"$OUT/make_fixtures_f64" "$HERE" "${1:-}"
