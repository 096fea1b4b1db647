"""Dose outputs (dpmx_result_write): the raw 3-D dose/uncertainty file and the
hist.sim-format depth profile for slab and voxel phantoms, checked against the
tallies they are made from."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def read_hist(path):
    rows = [l.split() for l in open(path) if not l.startswith("#")]
    return np.array([[float(x) for x in r] for r in rows])


def test_raw_round_trip(tables_wlb, dpm, tmp_path):
    from importlib import import_module
    wl = import_module("dpm-g4cpp_gb300.workloads")
    m = wl.precision_phantom(nx=24, ny=20, nz=32, v=3.0)
    ph = dpm.Phantom.voxels(tables_wlb, m, 3.0)
    n, B = 20000, 10
    r = dpm.run(tables_wlb, [dpm.Job(ph, wl.precision_source(field=40.0), n, 3)], batches=B)
    d, d2, _ = r.tally(0)
    r.write(tmp_path / "d.raw", fmt=dpm.DOSE_RAW)
    dose, rel, head = dpm.read_dose_raw(tmp_path / "d.raw")
    assert head["histories"] == n and head["batches"] == B and (head["nz"], head["ny"], head["nx"]) == m.shape
    rho = [tables_wlb.density(k) for k in range(tables_wlb.num_materials)]
    expect = wl.dose_gy(d, m, rho, 27.0, n)
    np.testing.assert_allclose(dose, expect, rtol=1e-6, atol=1e-30)
    sig = np.sqrt(np.maximum(d2 - d * d / B, 0.0) / (B - 1) * B)
    with np.errstate(divide="ignore", invalid="ignore"):
        er = np.where(d > 0, sig / d, 0.0)
    np.testing.assert_allclose(rel, er, rtol=1e-9, atol=1e-15)


def test_depth_profile_slab_matches_tally(tables_c3, dpm, tmp_path):
    ph = dpm.Phantom.slab(tables_c3, 3, 1.0)
    n = 20000
    r = dpm.run(tables_c3, [dpm.Job(ph, dpm.Source(particle=-1, e0=15.0, e1=15.0), n, 5)], batches=5)
    d, _, steps = r.tally(0)
    r.write(tmp_path / "hist.sim", fmt=dpm.DOSE_DEPTH)
    h = read_hist(tmp_path / "hist.sim")
    rho = np.array([tables_c3.density(0 if (iz < 10 or iz >= 25) else (1 if iz < 15 else 2)) for iz in range(len(h))])
    np.testing.assert_allclose(h[:, 1], (np.arange(len(h)) + 0.5) * 0.1, rtol=1e-4)
    np.testing.assert_allclose(h[:, 2], d[:len(h)] / (n * 0.1 * rho), rtol=1e-4, atol=1e-12)
    np.testing.assert_allclose(h[:, 3], steps[:len(h)] / n, rtol=1e-4, atol=1e-12)
    assert d[len(h):].sum() == 0.0


def test_depth_profile_voxels(tables_wlb, dpm, tmp_path):
    m = np.zeros((30, 8, 8), dtype=np.uint8)
    m[10:20] = 2                      # bone layer
    m[:, :, :2] = 1                   # lung strip: a slice of mixed density
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    n = 20000
    r = dpm.run(tables_wlb, [dpm.Job(ph, dpm.Source(particle=0, e0=6.0, e1=6.0, shape=1, fx=8.0, fy=8.0), n, 9)],
                batches=4)
    d, _, _ = r.tally(0)
    r.write(tmp_path / "depth.sim", fmt=dpm.DOSE_DEPTH)
    h = read_hist(tmp_path / "depth.sim")
    rho = np.array([tables_wlb.density(k) for k in range(3)])[m].mean(axis=(1, 2))
    assert len(h) == m.shape[0]
    np.testing.assert_allclose(h[:, 2], d.sum(axis=(1, 2)) / (n * 0.2 * rho), rtol=1e-4, atol=1e-12)
    assert not h[:, 3].any()


def test_result_outlives_its_phantom(tables_wlb, dpm, tmp_path):
    """a result keeps the material ids its dose outputs need: written after
    its phantom is freed and the device blocks have served another phantom
    and run, it gives the file written before"""
    m = np.zeros((20, 10, 10), dtype=np.uint8)
    m[5:10] = 2
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    r = dpm.run(tables_wlb, [dpm.Job(ph, dpm.Source(particle=-1, e0=8.0, e1=8.0, shape=1, fx=6.0, fy=6.0), 20000, 4)],
                batches=4)
    r.write(tmp_path / "before.raw", fmt=dpm.DOSE_RAW)
    ph.close()
    other = dpm.Phantom.voxels(tables_wlb, np.ones((20, 10, 10), dtype=np.uint8), 2.0)
    dpm.run(tables_wlb, [dpm.Job(other, dpm.Source(particle=0, e0=3.0, e1=3.0), 5000, 5)], batches=2).close()
    other.close()
    r.write(tmp_path / "after.raw", fmt=dpm.DOSE_RAW)
    a, ra, ha = dpm.read_dose_raw(tmp_path / "before.raw")
    b, rb, hb = dpm.read_dose_raw(tmp_path / "after.raw")
    assert a.sum() > 0.0 and ha == hb
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ra, rb)
