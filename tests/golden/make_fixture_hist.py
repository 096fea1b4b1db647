"""Writes fixture_hist_water_ti_bone_15MeV.npz from the reference's published
depth-dose fixture (tests/WaterTiBoneWater_15MeV/hist.sim of the reference: its
dpm_Simulate on Geant4-built data, 15 MeV e- pencil beam, water/Ti/bone/water
slabs of config 3, 1 mm bins). Columns: bin index, depth [cm], energy deposit
[MeV cm2/g] per history, scoring steps per history; plus the mean deposit.

    python tests/golden/make_fixture_hist.py [reference-root]   (default $DPM_REFERENCE_ROOT)
"""
import os
import sys

import numpy as np

ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DPM_REFERENCE_ROOT", "/root/reference")
src = os.path.join(ref, "tests", "WaterTiBoneWater_15MeV", "hist.sim")
rows, mean = [], None
for line in open(src):
    if line.startswith("# === Mean energy deposit"):
        mean = float(line.split(":")[1].split()[0])
    elif line.strip() and not line.startswith("#"):
        rows.append([float(v) for v in line.split()])
a = np.array(rows)
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fixture_hist_water_ti_bone_15MeV.npz")
np.savez(out, index=a[:, 0].astype(np.int32), depth_cm=a[:, 1], edep=a[:, 2], steps=a[:, 3], mean_edep=mean)
print(out, a.shape, mean)
