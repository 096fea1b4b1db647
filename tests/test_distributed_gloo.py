"""The multi-process path on CPU: history sharding covers every history once and
the tally reduction over two gloo ranks equals the unsharded tally (a
deterministic stand-in replaces the transport, so no GPU is needed)."""
import importlib
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def fake_tally(first, count, nbins=64):
    t = np.zeros(nbins)
    h = np.arange(first, first + count)
    np.add.at(t, h % nbins, np.sqrt(h + 1.0))
    return t


def _worker(rank, world, port, n, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    dd = importlib.import_module("dpm-g4cpp_gb300.distributed")
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, count = dd.shard(n, rank, world)
    total = dd.allreduce_sum(fake_tally(first, count))
    if rank == 0:
        np.save(out, total)
    dist.destroy_process_group()


@pytest.mark.parametrize("n", [1000, 1001, 7])
def test_shards_cover_histories_once(dpm, n):
    dd = importlib.import_module("dpm-g4cpp_gb300.distributed")
    for world in (1, 2, 3, 8):
        seen = np.zeros(n, dtype=int)
        for r in range(world):
            f, c = dd.shard(n, r, world)
            seen[f:f + c] += 1
        assert (seen == 1).all()


def test_gloo_two_ranks_sum_equals_unsharded(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "total.npy")
    n = 5003
    mp.spawn(_worker, args=(2, _free_port(), n, out), nprocs=2, join=True)
    np.testing.assert_allclose(np.load(out), fake_tally(0, n), rtol=1e-13)


def _failing_worker(rank, world, port, n, out_dir):
    import datetime
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    dd = importlib.import_module("dpm-g4cpp_gb300.distributed")
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    first, count = dd.shard(n, rank, world)
    status = "ok"
    try:
        if rank == 1:
            raise RuntimeError("planted failure before the reduction")
        dd.allreduce_sum(fake_tally(first, count))
    except Exception as e:    # the failure is what the test looks for
        status = "error: %s" % e
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write(status)
    os._exit(0)               # leave without the group's teardown: a failed rank does not join it


def test_a_failed_rank_ends_the_others_reduction(tmp_path):
    """a rank that fails between steps (it raises and leaves without joining
    the reduction) ends the other rank's reduction with an error, within the
    process group's timeout, instead of a hang"""
    import time
    import torch.multiprocessing as mp
    t0 = time.time()
    mp.spawn(_failing_worker, args=(2, _free_port(), 4000, str(tmp_path)), nprocs=2, join=True)
    assert time.time() - t0 < 120
    r1 = (tmp_path / "rank1.txt").read_text()
    r0 = (tmp_path / "rank0.txt").read_text()
    assert "planted failure" in r1
    assert r0.startswith("error"), r0
