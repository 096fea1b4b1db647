"""The drop-in CLI: same options and hist.sim layout as the reference
dpm_Simulate (dpm_Simulate.cc:35-45, Geom.cc:167-192)."""
import importlib
import os
import subprocess

import numpy as np
import pytest

from conftest import DATA_C3

pytestmark = pytest.mark.gpu


def read_hist(path):
    rows = [l.split() for l in open(path) if not l.startswith("#")]
    return np.array([[float(x) for x in r] for r in rows])


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_cli_writes_reference_format(tmp_path, tables_c3, dpm, prec):
    builder = importlib.import_module("dpm-g4cpp_gb300.builder")
    builder.build()
    out = tmp_path / "hist.sim"
    cmd = [os.path.join(builder.BINDIR, "dpm_simulate"), "-p", "e-", "-e", "15", "-n", "3000", "-d", DATA_C3,
           "-b", "1", "-c", "3", "-o", str(out), "-s", "321", "-P", prec]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    text = open(out).read().splitlines()
    assert text[0].startswith("# === Mean energy deposit in the target:")
    assert text[2].startswith("# === Index       Depth [cm]")
    h = read_hist(out)
    assert h.shape[1] == 4 and h.shape[0] >= 100
    assert np.allclose(h[:, 1], (np.arange(len(h)) + 0.5) * 0.1, rtol=1e-4)
    e, s = dpm.simulate(tables_c3, 3000, 15.0, True, 1.0, 3, seed=321,
                        precision=dpm.FP64_PLAIN if prec == "fp64" else dpm.FP32_EVENT)
    assert len(e) == len(h)
    dens = np.array([tables_c3.density(0 if i < 10 else (1 if i < 15 else (2 if i < 25 else 0))) for i in range(len(e))])
    np.testing.assert_allclose(h[:, 2], e / (3000 * 0.1) / dens, rtol=1e-3, atol=1e-7)
    mean = float(text[0].split(":")[1].split()[0])
    assert mean == pytest.approx(e.sum() / 3000, rel=1e-3)


def test_cli_bad_particle_exits_like_reference(tmp_path):
    builder = importlib.import_module("dpm-g4cpp_gb300.builder")
    p = subprocess.run([os.path.join(builder.BINDIR, "dpm_simulate"), "-p", "proton"], capture_output=True,
                       text=True, timeout=60)
    assert p.returncode == 255
    assert "Unknown primary particle name" in p.stdout


def test_cli_missing_data_dir(tmp_path):
    builder = importlib.import_module("dpm-g4cpp_gb300.builder")
    p = subprocess.run([os.path.join(builder.BINDIR, "dpm_simulate"), "-d", str(tmp_path / "nope"), "-n", "10"],
                       capture_output=True, text=True, timeout=60)
    assert p.returncode == 1
    assert "mat.dat" in p.stderr
