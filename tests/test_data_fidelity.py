"""Absolute physics of the generated data against the reference's only
published dose: its depth dose of a 15 MeV e- pencil beam in water/Ti/bone/water
(config 3, 1 mm bins) from Geant4-built data (tests/WaterTiBoneWater_15MeV/
hist.sim of the reference, 2e5 histories; tests/golden/make_fixture_hist.py).
The reference's own transport (restated by the oracle, pinned bit for bit to
the reference build) runs on this project's Geant4-free data, so what is tested
is the data generator: stopping powers, the density effect, elastic transport
cross sections. Region means of the dose ratio stay within 2.5 %, the depth of
50 % dose within 0.5 mm, the mean deposit within 1 %."""
import os

import numpy as np
import pytest

from conftest import DATA_C3, ROOT

FIXTURE = os.path.join(ROOT, "tests", "golden", "fixture_hist_water_ti_bone_15MeV.npz")


def densities(data_dir):
    with open(os.path.join(data_dir, "mat.dat")) as f:
        lines = f.read().splitlines()
    return [float(lines[i + 1].split()[2]) for i, l in enumerate(lines) if l.startswith("# Material index, name")]


def r50(dose, depth):
    i = int(np.argmax(dose))
    half = 0.5 * dose[i]
    j = i + int(np.argmax(dose[i:] < half))
    return depth[j - 1] + (depth[j] - depth[j - 1]) * (dose[j - 1] - half) / (dose[j - 1] - dose[j])


def test_depth_dose_matches_published_fixture(oracle_c3):
    fx = np.load(FIXTURE)
    n = 200000
    ed, _, _ = oracle_c3.simulate_slab(n, 15.0, True, 1.0, 3, seed=2024)
    rho = densities(DATA_C3)
    nb = min(len(ed), len(fx["edep"]))
    iz = np.arange(nb)
    mat = np.where(iz < 10, 0, np.where(iz < 15, 1, np.where(iz < 25, 2, 0)))   # config 3 slabs, 1 mm
    ours = ed[:nb] / n / (np.take(rho, mat) * 0.1)    # MeV cm2/g, as hist.sim
    ratio = ours[:45] / fx["edep"][:45]
    for a, b in ((0, 10), (10, 15), (15, 25), (25, 35), (35, 45)):
        assert abs(ratio[a:b].mean() - 1.0) < 0.025, (a, b, ratio[a:b].mean())
    assert abs(r50(ours, fx["depth_cm"][:nb]) - r50(fx["edep"][:nb], fx["depth_cm"][:nb])) < 0.05   # cm
    assert ed.sum() / n == pytest.approx(float(fx["mean_edep"]), rel=0.01)
