"""The allocation-free compaction entry point, through the C ABI.

pbf_launch_cell_ranges_compact_noalloc serves callers that cannot allocate
device memory while they run (a frame loop where cudaMalloc / cudaFree would
synchronize the device, a plugin host that hands out no GPU memory).  It keeps
its scratch in a fixed device array inside the library, shared by all calls.
This test runs it twice in a row on different inputs (the second call must
not see the first call's leftovers) and checks both results against the
allocating entry point, pbf_launch_cell_ranges_compact: the tables are
integer data, so they must be identical.  It also checks that a call beyond
the array's limit is refused without a launch.

The file is named to be collected last, so that a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import pbfx

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 24


def _tables(torch, lib, keys, noalloc):
    n = keys.size
    dks = torch.from_numpy(keys.view(np.int32)).cuda()
    uk = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    off = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    if noalloc:
        st = lib.pbf_launch_cell_ranges_compact_noalloc(P(uk), P(off), P(cnt), P(dks), n, None)
    else:
        sb = C.c_size_t()
        pbfx.check(lib.pbf_cell_compact_scratch_query(C.byref(sb), n))
        scratch = torch.empty(sb.value, dtype=torch.uint8, device="cuda")
        st = lib.pbf_launch_cell_ranges_compact(P(scratch), sb.value, P(uk), P(off), P(cnt), P(dks), n, None)
    pbfx.check(st, "compaction")
    torch.cuda.synchronize()
    m = int(cnt.cpu()[0])
    return m, uk.cpu().numpy()[:m].view(np.uint32).copy(), off.cpu().numpy()[: m + 1].view(np.uint32).copy()


def test_noalloc_matches_allocating_entry_point_on_two_calls(gpu, lib):
    torch = gpu
    rng = np.random.default_rng(7)
    for n, cells in ((300_001, 2_000_000), (5_000, 900)):
        keys = np.sort(rng.integers(0, cells, n).astype(np.uint32))
        m_ref, uk_ref, off_ref = _tables(torch, lib, keys, noalloc=False)
        m, uk, off = _tables(torch, lib, keys, noalloc=True)
        assert m == m_ref == len(np.unique(keys))
        np.testing.assert_array_equal(uk, uk_ref)
        np.testing.assert_array_equal(off, off_ref)


def test_noalloc_refuses_more_keys_than_its_array_holds(gpu, lib):
    st = lib.pbf_launch_cell_ranges_compact_noalloc(None, None, None, None, MAX_KEYS + 1, None)
    assert st == pbfx.PBF_ERR_UNSUPPORTED
