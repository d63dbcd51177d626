#!/bin/bash
# Regenerates the benchmark-size golden files (tests/golden/openmoc_*.json)
# by running OpenMOC's own FP64 CPUSolver on the benchmark configurations
# through oracle/openmoc_run.cpp: the 17 x 17 / 70-group assembly for 20
# source iterations and the 51 x 51 / 7-group core for 6.  Needs the OpenMOC
# source tree (REF=<tree>); run from the repo root:
#   REF=<OpenMOC source tree> bash tests/golden/make_config_goldens.sh
set -euo pipefail
: "${REF:?REF must name an OpenMOC source tree}"
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
OUT=$ROOT/oracle/_ref
make -s -f "$ROOT/oracle/ref.mk" REF="$REF" OUT="$OUT" -j"$(nproc)"
"$OUT/openmoc_run_f64" pin7 golden 20 "$HERE/openmoc_pin7_f64.json"
"$OUT/openmoc_run_f64" assembly70 golden 20 "$HERE/openmoc_assembly70_f64.json"
"$OUT/openmoc_run_f64" core51 golden 6 "$HERE/openmoc_core51_f64.json"
