"""dpmx_simulate_noalloc: the Simulate workload for callers that cannot let the
library allocate device memory (it keeps its scratch in a fixed device array
and writes into caller-owned device arrays). Checked through the C ABI against
the allocating entry point dpmx_simulate on the same inputs, twice in a row so
that leftovers of one call in the shared scratch would show in the next.
Collected last so that a failure here does not hide the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def call_noalloc(lib, tables, n, e, ise, lbox, geom, seed, bins):
    import torch
    edep = torch.zeros(bins, dtype=torch.float64, device="cuda")
    edep2 = torch.zeros(bins, dtype=torch.float64, device="cuda")
    steps = torch.zeros(bins, dtype=torch.float64, device="cuda")
    hl = C.c_int(0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.dpmx_simulate_noalloc(tables.handle, n, e, 1 if ise else 0, lbox, geom, seed, C.c_void_p(edep.data_ptr()),
                                   C.c_void_p(edep2.data_ptr()), C.c_void_p(steps.data_ptr()), bins, C.byref(hl),
                                   C.c_void_p(stream))
    assert rc == 0, lib.dpmx_last_error().decode()
    return edep.cpu().numpy(), edep2.cpu().numpy(), steps.cpu().numpy(), hl.value


CASES = [(True, 15.0, 1.0, 3, 2000, 41), (False, 12.0, 2.0, 0, 3000, 42)]


@pytest.mark.parametrize("first", [0, 1])
def test_noalloc_matches_allocating_entry_point(tables_c3, dpm, first):
    lib = dpm.library()
    order = CASES if first == 0 else CASES[::-1]
    for ise, e, lbox, geom, n, seed in order:       # two different calls in a row
        ref_e, ref_s = dpm.simulate(tables_c3, n, e, ise, lbox, geom, seed=seed, precision=dpm.FP64_PLAIN)
        ed, ed2, st, hl = call_noalloc(lib, tables_c3, n, e, ise, lbox, geom, seed, bins=512)
        assert hl == len(ref_e)
        np.testing.assert_allclose(ed[:hl], ref_e, rtol=1e-12, atol=1e-12)
        np.testing.assert_array_equal(st[:hl], ref_s)
        np.testing.assert_allclose(ed2[:hl], ref_e ** 2, rtol=1e-12, atol=1e-12)
        assert not ed[hl:].any() and not st[hl:].any()


def test_noalloc_at_the_smallest_voxel_size(tables_c3, dpm):
    """0.1 mm voxels: 1001 depth bins, close to the 1023-bin limit that both
    entry points share; a buffer of the full 8192 bins is accepted."""
    lib = dpm.library()
    for _ in range(2):
        ref_e, ref_s = dpm.simulate(tables_c3, 300, 15.0, True, 0.1, 3, seed=43, precision=dpm.FP64_PLAIN)
        ed, ed2, st, hl = call_noalloc(lib, tables_c3, 300, 15.0, True, 0.1, 3, 43, bins=8192)
        assert hl == len(ref_e) and hl > 900
        np.testing.assert_allclose(ed[:hl], ref_e, rtol=1e-12, atol=1e-12)
        np.testing.assert_array_equal(st[:hl], ref_s)


def test_noalloc_rejects_sizes_beyond_its_scratch(tables_c3, dpm):
    lib = dpm.library()
    import torch
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    rc = lib.dpmx_simulate_noalloc(tables_c3.handle, 10, 15.0, 1, 1.0, 3, 1, p, None, p, 8193, None, None)
    assert rc == dpm.ERR_ARG
    assert b"8192" in lib.dpmx_last_error()
    rc = lib.dpmx_simulate_noalloc(tables_c3.handle, 10, 15.0, 1, 1.0, 3, 1, p, None, p, 16, None, None)
    assert rc == dpm.ERR_ARG    # fewer bins than the 1 mm geometry needs
    # below 0.098 mm the slab geometry needs more than 1023 depth bins: both
    # entry points reject it
    rc = lib.dpmx_simulate_noalloc(tables_c3.handle, 10, 15.0, 1, 0.09, 3, 1, p, None, p, 8192, None, None)
    assert rc == dpm.ERR_ARG and b"too small" in lib.dpmx_last_error()
    with pytest.raises(dpm.DpmxError):
        dpm.simulate(tables_c3, 10, 15.0, True, 0.09, 3, seed=1)
