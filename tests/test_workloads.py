"""The synthetic workloads the benchmark and the measurements run, pinned to
the configurations they stand for: the precision phantom's water body, lung
slab and bone cylinder and its beam; the 64 batching jobs; the beamlet grid
and target of the differentiation form; the CT-like phantom (at a quarter of
its resolution, same extents)."""
import importlib
import math

import numpy as np

wl = importlib.import_module("dpm-g4cpp_gb300.workloads")


def test_precision_workload():
    m = wl.precision_phantom()
    assert m.shape == (256, 128, 128) and m.dtype == np.uint8
    assert set(np.unique(m)) == {wl.WATER, wl.LUNG, wl.BONE}
    z = (np.arange(256) + 0.5) * 2.0
    lung_planes = np.flatnonzero((m == wl.LUNG).any(axis=(1, 2)))
    assert z[lung_planes].min() > 60.0 and z[lung_planes].max() < 120.0 and len(lung_planes) == 30
    assert (m[lung_planes] == wl.LUNG).all()
    bone = m == wl.BONE
    assert (bone == bone[:, :1, :]).all()                     # a cylinder along y
    iz, ix = np.nonzero(bone[:, 0, :])
    x = (ix + 0.5) * 2.0 - 128.0
    assert abs(x.mean()) < 0.5 and abs(z[iz].mean() - 180.0) < 0.5
    assert abs(len(iz) * 4.0 / (math.pi * 15.0 ** 2) - 1.0) < 0.1
    s = wl.precision_source()
    assert (s.particle, s.spectrum, s.e0, s.e1, s.shape, s.fx, s.fy) == (0, 1, 1.0, 20.0, 1, 100.0, 100.0)


def test_batching_jobs():
    specs = [wl.batching_job_spec(i) for i in range(64)]
    edges = {m.shape[0] for m, _, _ in specs}
    assert edges <= {32, 64, 96, 128, 192} and len(edges) >= 3
    hist = np.array([h for _, _, h in specs])
    assert hist.min() >= 1e5 and hist.max() <= 1e7
    assert abs(hist.sum() / 1.37e8 - 1.0) < 0.01          # the 1.37e8 histories the measurements quote
    kinds = [s.particle for _, s, _ in specs]
    assert 16 < kinds.count(0) < 48
    assert all(4.0 <= s.e0 <= 20.0 and s.e0 == s.e1 for _, s, _ in specs)
    assert all(m.shape[0] == m.shape[1] == m.shape[2] for m, _, _ in specs)
    assert sum(len(np.unique(m)) > 1 for m, _, _ in specs) >= 60      # inserts in (almost) every phantom


def test_differentiation_setup():
    m, src, target = wl.differentiation_setup()
    assert m.shape == (128, 128, 128)
    assert {wl.WATER, wl.LUNG, wl.BONE} <= set(np.unique(m))
    assert (src.particle, src.e0, src.shape, src.nbx, src.nby, src.fx, src.fy) == (0, 6.0, 2, 20, 20, 5.0, 5.0)
    assert set(np.unique(target)) == {0.0, 2.0}
    vol = (target > 0).sum() * 8.0
    assert abs(vol / (4.0 / 3.0 * math.pi * 15.0 ** 3) - 1.0) < 0.1


def test_full_scale_phantom_structure():
    m = wl.full_scale_phantom(nx=128, ny=128, nz=64, v=4.0)
    assert set(np.unique(m)) == {wl.WATER, wl.LUNG, wl.BONE, wl.AIR}
    assert (m[0] == wl.AIR).all() and (m[:, :, 0] == wl.AIR).all()     # air around the body
    assert (m[32, 64, 64] != wl.AIR)
    s = wl.full_scale_source()
    assert (s.particle, s.spectrum, s.e0, s.e1, s.fx, s.fy) == (0, 2, 0.5, 20.0, 100.0, 100.0)
