"""Batching form: many independent jobs (different phantoms, particles,
energies, history counts) in one graph-captured run. A particle's trajectory
depends only on its own random stream (job seed, history, lineage), never on
which chunk, generation or lane transports it, so a batched run reproduces the
separate runs tally for tally up to the order of FP64 additions; so do runs with
other chunk sizes, launch shapes, without the graph, or split by history. (The
lane and block kernels of a phase are two forms: they round or draw random
numbers differently, so the choice of kernel is fixed for a run.)"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_jobs(dpm, tables, n=5):
    wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
    jobs, phantoms = wl.batching_jobs(tables, njobs=n, hist_range=(2e3, 2e4))
    return jobs, phantoms


def tallies(res, n):
    return [res.tally(j)[:2] for j in range(n)]


def assert_same(a, b, rtol=1e-10):
    for (d1, q1), (d2, q2) in zip(a, b):
        np.testing.assert_allclose(d1, d2, rtol=rtol, atol=1e-12 * max(1.0, d1.max()))
        np.testing.assert_allclose(q1, q2, rtol=rtol, atol=1e-12 * max(1.0, q1.max()))


def test_batched_equals_separate(tables_wlb, dpm):
    jobs, keep = small_jobs(dpm, tables_wlb)
    batched = dpm.run(tables_wlb, jobs, batches=4)
    sep = [dpm.run(tables_wlb, [j], batches=4).tally(0)[:2] for j in jobs]
    assert_same(tallies(batched, len(jobs)), sep)
    for j in range(len(jobs)):
        st = batched.stats(j)
        assert st.lost == 0 and st.residual_violations == 0
        assert st.histories == jobs[j].histories


def test_many_jobs_equal_separate(tables_wlb, dpm):
    """more jobs than the phase kernels keep in shared memory (16): their job
    records are read from global memory, with the same results"""
    jobs, keep = small_jobs(dpm, tables_wlb, n=20)
    batched = dpm.run(tables_wlb, jobs, batches=2)
    for j in (0, 7, 15, 16, 19):
        alone = dpm.run(tables_wlb, [jobs[j]], batches=2).tally(0)[:2]
        assert_same([batched.tally(j)[:2]], [alone])
        st = batched.stats(j)
        assert st.lost == 0 and st.residual_violations == 0 and st.histories == jobs[j].histories


def test_schedule_invariance(tables_wlb, dpm):
    jobs, keep = small_jobs(dpm, tables_wlb, n=3)
    base = tallies(dpm.run(tables_wlb, jobs, batches=2), 3)
    for kw in (dict(use_graph=False), dict(chunk_histories=3000), dict(block_size=128, blocks_per_sm=4),
               dict(tally_aggregate=1), dict(electron_slots=384)):
        r = dpm.run(tables_wlb, jobs, batches=2, **kw)
        if "electron_slots" in kw:
            assert r.config["electron_slots"] == 384
        assert_same(tallies(r, 3), base)


def test_chunk_lanes_equal_one_chunk(tables_wlb, dpm):
    """a run of 2^23 or more histories is cut into at least two chunks that
    run on two streams at once (chunk lanes); its tally equals the same job run
    as one chunk up to the order of FP64 additions"""
    wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
    ph = dpm.Phantom.voxels(tables_wlb, wl.precision_phantom(nx=64, ny=64, nz=128, v=4.0), 4.0)
    n = 8_400_000
    job = dpm.Job(ph, wl.precision_source(), n, 5)
    two = dpm.run(tables_wlb, [job], batches=2)
    assert two.config["chunk_histories"] == n // 2
    one = dpm.run(tables_wlb, [job], batches=2, chunk_histories=n)
    assert_same(tallies(two, 1), tallies(one, 1))
    for r in (one, two):
        st = r.stats(0)
        assert st.lost == 0 and st.residual_violations == 0 and st.histories == n


def test_autotuned_run_equals_its_configuration(tables_wlb, dpm):
    """the autotuner may pick the lane kernels, which draw other random numbers
    than the block kernels; a tuned run equals a plain run of the chosen shape"""
    jobs, keep = small_jobs(dpm, tables_wlb, n=3)
    tuned = dpm.run(tables_wlb, jobs, batches=2, autotune=True)
    c = tuned.config
    again = dpm.run(tables_wlb, jobs, batches=2, block_size=c["block_size"], blocks_per_sm=c["blocks_per_sm"],
                    tally_aggregate=c["tally_aggregate"], electron_kernel=c["electron_kernel"],
                    photon_kernel=c["photon_kernel"], chunk_histories=c["chunk_histories"],
                    electron_slots=c["electron_slots"])
    assert c["electron_slots"] in (384, 448)
    assert_same(tallies(tuned, 3), tallies(again, 3))
    for j in range(3):
        assert tuned.stats(j).lost == 0 and tuned.stats(j).residual_violations == 0


def test_history_split_sums_to_whole(tables_wlb, dpm):
    jobs, keep = small_jobs(dpm, tables_wlb, n=1)
    j = jobs[0]
    whole = dpm.run(tables_wlb, [j], batches=1).tally(0)[0]
    dd = importlib.import_module("dpm-g4cpp_gb300.distributed")
    parts = [dpm.run(tables_wlb, [dd.shard_job(j, r, 3)], batches=1).tally(0)[0] for r in range(3)]
    np.testing.assert_allclose(sum(parts), whole, rtol=1e-10, atol=1e-12 * whole.max())


def test_fp64_batched_matches_oracle_voxel(tables_wlb, oracle_wlb, dpm):
    """a small voxel job, FP64 form, history by history against the oracle:
    identical streams give identical histories except where a last-bit
    difference of a transcendental flips a branch; those are counted"""
    wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
    m = wl.precision_phantom(nx=24, ny=24, nz=48, v=5.0)
    ph = dpm.Phantom.voxels(tables_wlb, m, 5.0)
    src = wl.precision_source(field=60.0)
    n = 3000
    he, g = dpm.job_histories(tables_wlb, dpm.Job(ph, src, n, 77), with_dose=True)
    s = dict(particle=src.particle, spectrum=src.spectrum, e0=src.e0, e1=src.e1, shape=src.shape, cx=src.cx,
             cy=src.cy, fx=src.fx, fy=src.fy, nbx=src.nbx, nby=src.nby)
    o, ho, _ = oracle_wlb.simulate_voxel(m, 5.0, s, n, 77)
    same = np.isclose(he, ho, rtol=1e-9, atol=1e-12)
    assert (~same).sum() <= max(1, int(0.02 * n)), int((~same).sum())
    assert abs(he[same].sum() / ho[same].sum() - 1) < 1e-9
    # the run through dpmx_run gives the same dose as the per-history hook
    res = dpm.run(tables_wlb, [dpm.Job(ph, src, n, 77)], precision=dpm.FP64_PLAIN, batches=1)
    np.testing.assert_allclose(res.tally(0)[0].reshape(-1), g, rtol=1e-9, atol=1e-12 * g.max())


def test_largest_job_count(tables_wlb, dpm):
    """256 jobs in one run (the job field of a particle's sub-job has 8 bits;
    257 are refused): every job is complete, and jobs at both ends and in
    the middle equal the same job run alone"""
    ph = dpm.Phantom.voxels(tables_wlb, np.zeros((8, 8, 8), dtype=np.uint8), 2.0)
    jobs = [dpm.Job(ph, dpm.Source(particle=-1 if j % 2 else 0, e0=2.0 + (j % 7), e1=2.0 + (j % 7), shape=1,
                                   fx=8.0, fy=8.0), 300, 1000 + j) for j in range(256)]
    with pytest.raises(dpm.DpmxError) as e:
        dpm.run(tables_wlb, jobs + [jobs[0]], batches=2)
    assert e.value.code == dpm.ERR_ARG
    r = dpm.run(tables_wlb, jobs, batches=2)
    for j in range(256):
        st = r.stats(j)
        assert st.histories == 300 and st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
    for j in (0, 15, 16, 128, 255):
        alone = dpm.run(tables_wlb, [jobs[j]], batches=2).tally(0)[0]
        np.testing.assert_allclose(r.tally(j)[0], alone, rtol=1e-10, atol=1e-12 * max(1e-30, alone.max()))


@pytest.mark.parametrize("precision", [0, 1])
def test_concurrent_runs_from_threads(tables_wlb, dpm, precision):
    """runs made at once from four host threads (each on its own stream, with
    its own executable graph; the scratch pool lends a block to one run at a
    time) give the doses of the same runs made one after another"""
    from concurrent.futures import ThreadPoolExecutor
    m = np.zeros((32, 16, 16), dtype=np.uint8)
    m[10:14] = 2
    ph = dpm.Phantom.voxels(tables_wlb, m, 2.0)
    n = 4000 if precision == dpm.FP64_PLAIN else 200000
    jobs = [dpm.Job(ph, dpm.Source(particle=k % 2 - 1, e0=4.0 + k, e1=4.0 + k, shape=1, fx=12.0, fy=12.0), n, 70 + k)
            for k in range(8)]

    def one(job):
        r = dpm.run(tables_wlb, [job], precision=precision, batches=4)
        d = r.tally(0)[0]
        r.close()
        return d

    seq = [one(j) for j in jobs]
    with ThreadPoolExecutor(4) as ex:
        par = list(ex.map(one, jobs))
    for a, b in zip(seq, par):
        assert a.sum() > 0.0
        np.testing.assert_allclose(b, a, rtol=1e-10, atol=1e-12 * a.max())
