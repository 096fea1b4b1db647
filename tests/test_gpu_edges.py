"""Edge cases and size-independent properties of the FP32 event form.

* empty and ragged jobs (0 histories, fewer histories than batches);
* vacuum voxels end every track that reaches them (SimDPMLike.cc:88-93,
  :282-287, :495-500), so nothing is scored behind a vacuum layer;
* the block-local depth tally of slab jobs gives the same dose as global
  atomics (a history's deposits do not depend on the batching);
* phantoms at the largest dimensions (2047 x 2047 x 1023 voxels: the packed
  voxel index), beams into their last column and through their last planes;
  voxels of 0.05 and 20 mm; history indices up to 2^32 - 1; sources at the
  ends of the data set's energy range and every spectrum form; 65536
  statistical batches; a pencil beam along the faces between voxel columns;
* the full-size precision workload (128x128x256 x 2 mm, 1e7 histories):
  every history conserves energy, nothing is lost, and the FP32 dose agrees
  with the FP64 plain form within statistics.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_empty_and_ragged_jobs(tables_wlb, dpm):
    m = np.zeros((16, 16, 16), dtype=np.uint8)
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    src = dpm.Source(particle=0, e0=5.0, e1=5.0, shape=1, fx=10.0, fy=10.0)
    jobs = [dpm.Job(ph, src, 0, 1), dpm.Job(ph, src, 1, 2), dpm.Job(ph, src, 7, 3), dpm.Job(ph, src, 1000, 4)]
    r = dpm.run(tables_wlb, jobs, batches=10)
    d0, q0, _ = r.tally(0)
    assert not d0.any() and not q0.any()
    for j, job in enumerate(jobs):
        st = r.stats(j)
        assert st.histories == job.histories
        assert st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * max(1.0, st.primary_energy)
    # each job equals the same job run alone
    for j in (1, 2, 3):
        alone = dpm.run(tables_wlb, [jobs[j]], batches=10).tally(0)[0]
        np.testing.assert_allclose(r.tally(j)[0], alone, rtol=1e-10, atol=1e-12 * max(1.0, alone.max()))


def test_vacuum_layer_ends_tracks(tables_wlb, dpm):
    m = np.zeros((40, 16, 16), dtype=np.uint8)
    ph_water = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    m[10:12] = 255                      # vacuum layer at z = 20..24 mm
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    src = dpm.Source(particle=-1, e0=10.0, e1=10.0, shape=0)
    r = dpm.run(tables_wlb, [dpm.Job(ph, src, 20000, 5)], batches=5)
    w = dpm.run(tables_wlb, [dpm.Job(ph_water, src, 20000, 5)], batches=5)
    d, dw = r.tally(0)[0], w.tally(0)[0]
    st = r.stats(0)
    assert not d[10:12].any()           # nothing is scored in vacuum
    # no electron crosses the layer: behind it only bremsstrahlung photons
    # (which can step over it, Woodcock tracking) deposit energy
    assert d[12:16].sum() < 0.2 * dw[12:16].sum()
    assert st.lost == 0 and st.residual_violations == 0
    assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy


def test_all_vacuum_phantom(tables_wlb, dpm):
    m = np.full((8, 8, 8), 255, dtype=np.uint8)
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    r = dpm.run(tables_wlb, [dpm.Job(ph, dpm.Source(particle=0, e0=3.0, e1=3.0), 500, 6)], batches=2)
    st = r.stats(0)
    assert st.edep == 0.0
    assert abs(st.escaped - 500 * 3.0) < 1e-6
    assert st.histories == 500


def test_block_depth_tally_equals_global(tables_c3, dpm):
    ph = dpm.Phantom.slab(tables_c3, 3, 1.0)
    src = dpm.Source(particle=-1, e0=15.0, e1=15.0)
    # 10 batches x 101 bins fit the block-local depth tally; 20 do not
    a = dpm.run(tables_c3, [dpm.Job(ph, src, 20000, 77)], batches=10)
    b = dpm.run(tables_c3, [dpm.Job(ph, src, 20000, 77)], batches=20)
    da, _, sa = a.tally(0)
    db, _, sb = b.tally(0)
    np.testing.assert_allclose(da, db, rtol=1e-10, atol=1e-12 * da.max())
    np.testing.assert_array_equal(sa, sb)


def test_precision_workload_full_size(tables_wlb, dpm):
    from importlib import import_module
    wl = import_module("dpm-g4cpp_gb300.workloads")
    m = wl.precision_phantom()
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    src = wl.precision_source()
    n32, n64 = 10**7, 10**6
    r32 = dpm.run(tables_wlb, [dpm.Job(ph, src, n32, 7)], batches=10)
    st = r32.stats(0)
    assert st.lost == 0 and st.residual_violations == 0 and st.histories == n32
    assert abs(st.edep + st.escaped - st.primary_energy) < 1e-6 * st.primary_energy
    r64 = dpm.run(tables_wlb, [dpm.Job(ph, src, n64, 8)], precision=dpm.FP64_PLAIN, batches=10)
    d32, q32, _ = r32.tally(0)
    d64, q64, _ = r64.tally(0)
    # depth-dose profiles (summed over x, y) per history, with batch errors
    def profile(d, q, n):
        pz = d.sum(axis=(1, 2)) / n
        # the batch sums of a profile bin are not kept; bound its error by the
        # sum of the voxel errors (an overestimate, so the test stays fair)
        sz = np.sqrt(np.maximum(q * 10 - d * d, 0.0) / 9).sum(axis=(1, 2)) / n
        return pz, sz
    p32, s32 = profile(d32, q32, n32)
    p64, s64 = profile(d64, q64, n64)
    mask = p64 > 0.1 * p64.max()
    rel = (p32[mask] - p64[mask]) / p64[mask]
    assert np.abs(rel).mean() < 0.01, np.abs(rel).mean()
    assert (np.abs(p32[mask] - p64[mask]) <= 2 * np.sqrt(s32[mask] ** 2 + s64[mask] ** 2)).mean() >= 0.95
    assert abs(d32.sum() / n32 / (d64.sum() / n64) - 1.0) < 0.005


@pytest.mark.parametrize("kind", ["photon", "electron"])
def test_photon_kernels_give_the_same_histories(tables_wlb, dpm, kind):
    """the lane and the block-batched photon phase draw the same random numbers
    per photon: the same histories, up to FP32 rounding (the compiler contracts
    the same formulas differently in the two kernels) and summation order"""
    from importlib import import_module
    wl = import_module("dpm-g4cpp_gb300.workloads")
    m = wl.precision_phantom(nx=32, ny=32, nz=64, v=4.0)
    ph = dpm.Phantom.voxels(tables_wlb, m, 4.0)
    src = wl.precision_source(field=60.0) if kind == "photon" else dpm.Source(particle=-1, e0=12.0, e1=12.0, shape=1,
                                                                              fx=40.0, fy=40.0)
    a = dpm.run(tables_wlb, [dpm.Job(ph, src, 100000, 13)], batches=4, photon_kernel=0).tally(0)[0]
    b = dpm.run(tables_wlb, [dpm.Job(ph, src, 100000, 13)], batches=4, photon_kernel=1).tally(0)[0]
    assert abs(a.sum() / b.sum() - 1.0) < 1e-5
    close = np.isclose(a, b, rtol=1e-4, atol=1e-9 * a.max())
    assert close.mean() > 0.999, close.mean()


@pytest.mark.parametrize("shape", [(16, 16, 16), (7, 5, 3), (1, 1, 1), (33, 17, 9), (40, 512, 512)])
def test_material_ids_checked_on_upload(tables_wlb, dpm, shape):
    """ids beyond the data set are refused wherever they sit (also in the
    last bytes of an array whose size is no multiple of 16, and in an array
    of 10.5M voxels, where each thread of the check reads several 16-byte
    words); vacuum is not"""
    nmat = tables_wlb.num_materials
    m = np.zeros(shape, dtype=np.uint8)
    m.reshape(-1)[-1] = 255
    dpm.Phantom.voxels(tables_wlb, m, 2.0).close()
    m.reshape(-1)[-1] = nmat - 1
    dpm.Phantom.voxels(tables_wlb, m, 2.0).close()
    for pos in (0, m.size // 2, m.size - 1):
        bad = np.zeros(shape, dtype=np.uint8)
        bad.reshape(-1)[pos] = nmat
        with pytest.raises(dpm.DpmxError) as e:
            dpm.Phantom.voxels(tables_wlb, bad, 2.0)
        assert e.value.code == dpm.ERR_ARG


@pytest.mark.parametrize("shape,particle", [((1023, 2, 2047), 0), ((2, 2047, 2047), -1)])
def test_largest_phantom_dimensions(tables_wlb, dpm, shape, particle):
    """phantoms at the largest dimensions (2047 voxels in x and y, 1023 in z:
    the 11/11/10-bit packed voxel index of the queues and slots), a 10 MeV
    pencil beam into the last column (x = 2046, and y = 2046 on the wide
    phantom): photons through 1023 planes, electrons through 2. Both forms
    conserve energy, lose nothing, score in the beam's column (and, on the
    deep phantom, in its last planes) and agree on the deposited energy."""
    nz, ny, nx = shape
    ph = dpm.Phantom.voxels(tables_wlb, np.zeros(shape, dtype=np.uint8), 1.0)
    cx = 0.5 * nx - 0.5                                           # centre of column nx - 1 [mm]
    cy = 0.5 * ny - 0.5 if ny > 2 else 0.0
    src = dpm.Source(particle=particle, e0=10.0, e1=10.0, shape=0, cx=cx, cy=cy)
    n = 20000
    edep = {}
    for prec in (dpm.FP64_PLAIN, dpm.FP32_EVENT):
        r = dpm.run(tables_wlb, [dpm.Job(ph, src, n, 21)], precision=prec, batches=4)
        st = r.stats(0)
        assert st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
        d = r.tally(0)[0].reshape(shape)
        assert d.sum() > 0.0
        assert d[:, :, nx - 3:].sum() > 0.5 * d.sum()            # the beam's column and its neighbours
        if ny > 2:
            assert d[:, ny - 3:, :].sum() > 0.5 * d.sum()
        if nz > 2:
            assert d[nz - 24:].sum() > 0.0                       # the beam reaches the last planes
        edep[prec] = st.edep / n
    # the two forms' mean deposits per history agree within a few standard
    # errors (the deposit of one history lies in [0, 10] MeV)
    assert abs(edep[dpm.FP32_EVENT] - edep[dpm.FP64_PLAIN]) < 4 * 10.0 * np.sqrt(2.0 / n)


def test_history_index_range(tables_wlb, dpm):
    """a history's index is the counter of its random streams, so indices lie
    in [0, 2^32): jobs beyond are refused; the last 2000 indices run in both
    forms, and split into two jobs they give the one job's dose (the FP64
    form to summation order, the FP32 form within its rounding)"""
    m = np.zeros((24, 12, 12), dtype=np.uint8)
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    src = dpm.Source(particle=0, e0=6.0, e1=6.0, shape=1, fx=10.0, fy=10.0)
    top = 2 ** 32
    for bad in (dict(histories=1001, first_history=top - 1000), dict(histories=-1), dict(histories=10, first_history=-5)):
        with pytest.raises(dpm.DpmxError) as e:
            dpm.run(tables_wlb, [dpm.Job(ph, src, seed=3, **bad)])
        assert e.value.code == dpm.ERR_ARG
    for prec in (dpm.FP64_PLAIN, dpm.FP32_EVENT):
        one = dpm.run(tables_wlb, [dpm.Job(ph, src, 2000, 3, first_history=top - 2000)], precision=prec, batches=2)
        two = dpm.run(tables_wlb, [dpm.Job(ph, src, 1000, 3, first_history=top - 2000),
                                   dpm.Job(ph, src, 1000, 3, first_history=top - 1000)], precision=prec, batches=1)
        st = one.stats(0)
        assert st.histories == 2000 and st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
        d1 = one.tally(0)[0]
        d2 = two.tally(0)[0] + two.tally(1)[0]
        assert d1.sum() > 0.0
        tol = 1e-10 if prec == dpm.FP64_PLAIN else 1e-4
        np.testing.assert_allclose(d2, d1, rtol=tol, atol=tol * d1.max())


@pytest.mark.parametrize("v,e,shape", [(0.05, 2.0, (40, 12, 12)), (20.0, 12.0, (12, 6, 6))])
def test_voxel_size_extremes(tables_wlb, dpm, v, e, shape):
    """0.05 mm voxels (a 2 MeV electron crosses dozens in one condensed-history
    step: the FP32 form's voxel-local offsets and boundary pushes at their
    finest) and 20 mm voxels (a 12 MeV electron's track fits in three): the
    FP32 form's dose agrees with the FP64 form's voxel by voxel"""
    from importlib import import_module
    dc = import_module("dpm-g4cpp_gb300.dosecheck")
    ph = dpm.Phantom.voxels(tables_wlb, np.zeros(shape, dtype=np.uint8), v)
    src = dpm.Source(particle=-1, e0=e, e1=e)
    est = {}
    for prec, n in ((dpm.FP64_PLAIN, 40000), (dpm.FP32_EVENT, 400000)):
        r = dpm.run(tables_wlb, [dpm.Job(ph, src, n, 8)], precision=prec, batches=10)
        st = r.stats(0)
        assert st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
        d, q, _ = r.tally(0)
        est[prec] = dc.batch_estimate(d, q, 10, n)
    m32, s32 = est[dpm.FP32_EVENT]
    m64, s64 = est[dpm.FP64_PLAIN]
    c = dc.compare(m32, s32, 10, m64, s64, 10)
    assert c["voxels"] >= 10
    assert c["within_2sigma"] > 0.88, c
    assert abs(c["mean_signed_pct"]) < 1.0, c


@pytest.mark.parametrize("particle,spectrum,e0,e1", [
    (0, 0, 0.0501, 0.0501),    # photons just above the photon cut (0.05 MeV)
    (0, 0, 20.99, 20.99),      # photons just below the top of the tables (21 MeV)
    (-1, 0, 0.2001, 0.2001),   # electrons just above the electron cut (0.2 MeV)
    (-1, 0, 20.99, 20.99),     # electrons just below the top of the tables
    (0, 2, 0.5, 20.0),         # falling spectrum p(E) ~ (e1 - E)
    (-1, 1, 20.0, 1.0),        # uniform spectrum given high to low
])
def test_source_energy_extremes(tables_wlb, dpm, particle, spectrum, e0, e1):
    """sources at the ends of the data set's energy range and the other
    spectrum forms: both forms conserve every history's energy, lose
    nothing, and agree on the mean deposit per history"""
    ph = dpm.Phantom.voxels(tables_wlb, np.zeros((64, 32, 32), dtype=np.uint8), 2.0)
    src = dpm.Source(particle=particle, spectrum=spectrum, e0=e0, e1=e1, shape=1, fx=20.0, fy=20.0)
    mean = {}
    for prec, n in ((dpm.FP64_PLAIN, 20000), (dpm.FP32_EVENT, 200000)):
        r = dpm.run(tables_wlb, [dpm.Job(ph, src, n, 17)], precision=prec, batches=4)
        st = r.stats(0)
        assert st.histories == n and st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
        assert st.edep > 0.0
        mean[prec] = st.edep / n
    # a history deposits between 0 and its energy: sd <= max(e0, e1) / 2
    se = 0.5 * max(e0, e1) * np.sqrt(1.0 / 20000 + 1.0 / 200000)
    assert abs(mean[dpm.FP32_EVENT] - mean[dpm.FP64_PLAIN]) < 5.0 * se, (mean, se)


def test_largest_batch_count(tables_wlb, dpm):
    """65536 statistical batches (the most a run takes; 65537 is refused) on
    a small phantom, two histories per batch: both forms run them, the dose
    is the sum of the batch tallies (dose^2 >= dose^2 / batches bin by bin),
    and the FP32 dose equals the same job run in 4 batches up to FP64
    summation order (a history's deposits do not depend on its batch)"""
    ph = dpm.Phantom.voxels(tables_wlb, np.zeros((8, 8, 8), dtype=np.uint8), 2.0)
    src = dpm.Source(particle=-1, e0=5.0, e1=5.0, shape=1, fx=8.0, fy=8.0)
    B = 65536
    with pytest.raises(dpm.DpmxError) as e:
        dpm.run(tables_wlb, [dpm.Job(ph, src, 1000, 4)], batches=B + 1)
    assert e.value.code == dpm.ERR_ARG
    for prec in (dpm.FP64_PLAIN, dpm.FP32_EVENT):
        r = dpm.run(tables_wlb, [dpm.Job(ph, src, 2 * B, 4)], precision=prec, batches=B)
        st = r.stats(0)
        assert st.histories == 2 * B and st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
        d, q, _ = r.tally(0)
        assert d.sum() > 0.0
        assert np.all(q >= d * d / B * (1.0 - 1e-9))
        few = dpm.run(tables_wlb, [dpm.Job(ph, src, 2 * B, 4)], precision=prec, batches=4).tally(0)[0]
        np.testing.assert_allclose(d, few, rtol=1e-9, atol=1e-12 * few.max())


@pytest.mark.parametrize("particle,e", [(-1, 6.0), (0, 6.0)])
def test_pencil_beam_on_a_voxel_face(tables_wlb, dpm, particle, e):
    """a pencil beam at x = y = 0 of a phantom with an even number of voxels
    runs along the faces between four voxel columns: both forms put the
    particle in the same column (the one above the face) and agree voxel by
    voxel"""
    from importlib import import_module
    dc = import_module("dpm-g4cpp_gb300.dosecheck")
    ph = dpm.Phantom.voxels(tables_wlb, np.zeros((30, 16, 16), dtype=np.uint8), 2.0)
    src = dpm.Source(particle=particle, e0=e, e1=e)
    est, cols = {}, {}
    for prec, n in ((dpm.FP64_PLAIN, 40000), (dpm.FP32_EVENT, 400000)):
        r = dpm.run(tables_wlb, [dpm.Job(ph, src, n, 12)], precision=prec, batches=10)
        st = r.stats(0)
        assert st.lost == 0 and st.residual_violations == 0
        d, q, _ = r.tally(0)
        est[prec] = dc.batch_estimate(d, q, 10, n)
        first = d.reshape(30, 16, 16)[0]
        cols[prec] = np.unravel_index(first.argmax(), first.shape)
    assert cols[dpm.FP32_EVENT] == cols[dpm.FP64_PLAIN], cols
    c = dc.compare(est[dpm.FP32_EVENT][0], est[dpm.FP32_EVENT][1], 10,
                   est[dpm.FP64_PLAIN][0], est[dpm.FP64_PLAIN][1], 10)
    assert c["within_2sigma"] > 0.85, c
    assert abs(c["mean_signed_pct"]) < max(0.5, 3.0 * c["mean_rel_sigma_pct"]), c
