#!/usr/bin/env bash
# Builds the reference's simulation phase, unmodified, from its own sources
# (no Geant4 is needed on this side), into oracle/_ref/:
#   libdpm_ref.so  : Simulation/src/*.cc + oracle/ref_shim.cc (C entry points)
#   dpm_Simulate   : the reference CLI (dpm_Simulate.cc), glibc getopt_long
# The outputs are test infrastructure only (golden vectors, oracle pinning).
# Usage: oracle/build_ref.sh [reference-root]
#   (default $DPM_REFERENCE_ROOT, else the build container's mount point)
set -euo pipefail
REF="${1:-${DPM_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/Simulation/src" ]; then
  echo "reference sources not found under $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
CXXFLAGS="-O2 -std=c++11 -ffp-contract=off -w"
g++ $CXXFLAGS -fPIC -shared -I"$REF" -I"$REF/Simulation/inc" \
    "$REF"/Simulation/src/*.cc "$HERE/ref_shim.cc" -o "$OUT/libdpm_ref.so"
g++ $CXXFLAGS -I"$REF" -I"$REF/Simulation/inc" \
    "$REF/dpm_Simulate.cc" "$REF"/Simulation/src/*.cc -o "$OUT/dpm_Simulate"
echo "built $OUT/libdpm_ref.so and $OUT/dpm_Simulate"
