"""Per-voxel densities (Geom::GetVoxelMaterialDensity(iVoxel), Geom.hh:75-92):
nominal densities reproduce the plain phantom; scaled densities in the FP64
form agree with the oracle history by history, and the FP32 form agrees with
FP64 within statistics."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _src_dict(src):
    return dict(particle=src.particle, spectrum=src.spectrum, e0=src.e0, e1=src.e1, shape=src.shape, cx=src.cx,
                cy=src.cy, fx=src.fx, fy=src.fy, nbx=src.nbx, nby=src.nby)


def _phantom():
    m = np.zeros((40, 16, 16), dtype=np.uint8)
    m[12:20] = 2                                   # bone slab
    rho = np.ones(m.shape, dtype=np.float32)
    rho[m == 2] = 1.85
    rho[4:10] = 0.5                                # low-density water
    rho[24:30] = 1.6                               # water denser than nominal: majorant scaled
    return m, rho


@pytest.mark.parametrize("precision", [0, 1])
def test_nominal_density_reproduces_plain(tables_wlb, dpm, precision):
    m = np.zeros((24, 12, 12), dtype=np.uint8)    # water: its density 1.0 is exact in float
    src = dpm.Source(particle=0, e0=8.0, e1=8.0, shape=1, fx=10.0, fy=10.0)
    a = dpm.run(tables_wlb, [dpm.Job(dpm.Phantom.voxels(tables_wlb, m, 2.0), src, 20000, 3)], precision=precision)
    b = dpm.run(tables_wlb, [dpm.Job(dpm.Phantom.voxels(tables_wlb, m, 2.0, density=np.ones(m.shape, np.float32)),
                                     src, 20000, 3)], precision=precision)
    np.testing.assert_allclose(a.tally(0)[0], b.tally(0)[0], rtol=1e-10, atol=1e-12)


def test_nominal_densities_reproduce_plain_materials(tables_wlb, dpm):
    """three materials at their nominal densities given per voxel: the run
    takes the kernels' general geometry form (densities from the voxel array,
    spline descriptors per material from shared memory) and must equal the
    plain form of the same phantom (densities by material, descriptors of
    material 0 moved by a fixed stride) up to the order of FP64 additions"""
    m = np.zeros((32, 12, 12), dtype=np.uint8)
    m[8:16] = 1                                    # lung
    m[20:26] = 2                                   # bone
    rho = np.zeros(m.shape, dtype=np.float32)
    for k in range(3):
        rho[m == k] = np.float32(tables_wlb.density(k))
    src = dpm.Source(particle=0, e0=10.0, e1=10.0, shape=1, fx=10.0, fy=10.0)
    a = dpm.run(tables_wlb, [dpm.Job(dpm.Phantom.voxels(tables_wlb, m, 2.0), src, 50000, 9)])
    b = dpm.run(tables_wlb, [dpm.Job(dpm.Phantom.voxels(tables_wlb, m, 2.0, density=rho), src, 50000, 9)])
    (da, qa, _), (db, qb, _) = a.tally(0), b.tally(0)
    assert da.sum() > 0
    np.testing.assert_allclose(da, db, rtol=1e-10, atol=1e-12 * da.max())
    np.testing.assert_allclose(qa, qb, rtol=1e-10, atol=1e-12 * qa.max())


def test_fp64_density_matches_oracle(tables_wlb, oracle_wlb, dpm):
    m, rho = _phantom()
    src = dpm.Source(particle=-1, e0=12.0, e1=12.0, shape=1, fx=12.0, fy=12.0)
    n = 3000
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0, density=rho)
    g = dpm.run(tables_wlb, [dpm.Job(ph, src, n, 21)], precision=dpm.FP64_PLAIN, batches=1).tally(0)[0]
    o, _, _ = oracle_wlb.simulate_voxel(m, 2.0, _src_dict(src), n, 21, density=rho)
    assert abs(g.sum() / o.sum() - 1) < 2e-3
    close = np.isclose(g, o, rtol=1e-6, atol=1e-9 * o.max())
    assert close.mean() > 0.8, close.mean()


def test_fp32_density_matches_fp64(tables_wlb, dpm):
    m, rho = _phantom()
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0, density=rho)
    src = dpm.Source(particle=0, e0=10.0, e1=10.0, shape=1, fx=12.0, fy=12.0)
    n32, n64 = 20_000_000, 4_000_000
    a = dpm.run(tables_wlb, [dpm.Job(ph, src, n32, 1)], batches=10)
    b = dpm.run(tables_wlb, [dpm.Job(ph, src, n64, 2)], precision=dpm.FP64_PLAIN, batches=10)
    st = a.stats(0)
    assert st.lost == 0 and st.residual_violations == 0
    pa = a.tally(0)[0].sum(axis=(1, 2)) / n32
    pb = b.tally(0)[0].sum(axis=(1, 2)) / n64
    mask = pb > 0.1 * pb.max()
    assert np.abs(pa[mask] / pb[mask] - 1).mean() < 0.01
    # the dense and light layers change the depth dose: the density is used
    plain = dpm.run(tables_wlb, [dpm.Job(dpm.Phantom.voxels(tables_wlb, m, 2.0), src, n32, 2)], batches=10)
    pp = plain.tally(0)[0].sum(axis=(1, 2)) / n32
    # half density: about half the energy per slice, less in the build-up region
    # where fewer secondaries are set in motion upstream as well
    assert 1.5 < pp[4:10].sum() / pa[4:10].sum() < 3.5


def test_density_validation(tables_wlb, dpm):
    m = np.zeros((4, 4, 4), dtype=np.uint8)
    bad = np.zeros(m.shape, dtype=np.float32)
    with pytest.raises(dpm.DpmxError):
        dpm.Phantom.voxels(tables_wlb, m, 2.0, density=bad)


@pytest.mark.parametrize("particle,e", [(0, 6.0), (-1, 10.0)])
def test_density_extremes(tables_wlb, dpm, particle, e):
    """water layers at 0.001 and 10 g/cm3 (a Woodcock majorant scaled by 10,
    electron steps hundreds of voxels long in the thin layer): the FP32 form
    agrees with the FP64 form voxel by voxel, and both conserve energy"""
    dc = importlib.import_module("dpm-g4cpp_gb300.dosecheck")
    m = np.zeros((48, 12, 12), dtype=np.uint8)
    rho = np.ones(m.shape, dtype=np.float32)
    rho[6:18] = 0.001
    rho[30:36] = 10.0
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0, density=rho)
    src = dpm.Source(particle=particle, e0=e, e1=e, shape=1, fx=6.0, fy=6.0)
    est = {}
    for prec, n in ((dpm.FP64_PLAIN, 40000), (dpm.FP32_EVENT, 400000)):
        r = dpm.run(tables_wlb, [dpm.Job(ph, src, n, 31)], precision=prec, batches=10)
        st = r.stats(0)
        assert st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
        d, q, _ = r.tally(0)
        est[prec] = dc.batch_estimate(d, q, 10, n)
    c = dc.compare(est[dpm.FP32_EVENT][0], est[dpm.FP32_EVENT][1], 10,
                   est[dpm.FP64_PLAIN][0], est[dpm.FP64_PLAIN][1], 10)
    assert c["voxels"] >= 20
    assert c["within_2sigma"] > 0.88, c
    assert abs(c["mean_signed_pct"]) < 1.0, c
