#!/bin/sh
# Regenerates the data sets of this directory with the project's Geant4-free
# generator (dpm-g4cpp_gb300/bin/dpm_generate_data, built by build()). The
# Seltzer-Berger tables are read from the reference's SBTables/data (argument 1;
# default: SBTables/data under $DPM_REFERENCE_ROOT).
set -e
cd "$(dirname "$0")"
GEN=../dpm-g4cpp_gb300/bin/dpm_generate_data
SB=${1:-${DPM_REFERENCE_ROOT:-/root/reference}/SBTables/data}
mkdir -p water_ti_bone water_lung_bone water_lung_bone_air
"$GEN" -d water_ti_bone -c 3 -s "$SB" > /dev/null
"$GEN" -d water_lung_bone -c 6 -s "$SB" > /dev/null
"$GEN" -d water_lung_bone_air -c 6 -s "$SB" -m G4_WATER,G4_LUNG_ICRP,G4_BONE_COMPACT_ICRU,G4_AIR > /dev/null
