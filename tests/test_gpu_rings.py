"""The slot rings of the block-batched phases (bounded MPMC queues in shared
memory, one cell per position with a lap tag) on the GPU: every slot put on a
ring is taken exactly once per put, under eight warps per block contending for
the same rings, for slot counts from one to a full ring; and a wait on a cell
that nothing fills runs out after its bound and is reported, with the context
still usable afterwards."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nslots", [1, 31, 32, 33, 257, 352, 416, 512])
def test_every_slot_taken_once_per_put(dpm, gpu_lib, nslots):
    blocks, rounds = 64, 300
    taken, bad, gave_up, probes = dpm.ring_selftest(blocks=blocks, nslots=nslots, rounds=rounds, seed=nslots)
    assert gave_up == 0
    assert bad == 0
    assert taken == blocks * nslots * rounds
    assert probes == blocks


def test_many_laps_full_gpu(dpm, gpu_lib):
    # 152 x 3 blocks (the electron phase's grid) each lap a ring ~2000 times
    blocks, nslots, rounds = 456, 416, 2500
    taken, bad, gave_up, probes = dpm.ring_selftest(blocks=blocks, nslots=nslots, rounds=rounds, seed=99)
    assert (taken, bad, gave_up, probes) == (blocks * nslots * rounds, 0, 0, blocks)


def test_bounded_wait_reports_and_context_survives(dpm, tables_c3):
    # a probe bound of ~1 ms of clock cycles: each block's wait runs out
    assert dpm.ring_selftest(blocks=8, nslots=64, rounds=10, probe_cycles=2_000_000)[3] == 8
    # the context is intact: a transport run afterwards completes normally
    ph = dpm.Phantom.slab(tables_c3, 3, 1.0)
    r = dpm.run(tables_c3, [dpm.Job(ph, dpm.Source(particle=-1, e0=15.0, e1=15.0), 20000, 3)], batches=5)
    st = r.stats(0)
    assert st.histories == 20000 and st.lost == 0 and st.residual_violations == 0

