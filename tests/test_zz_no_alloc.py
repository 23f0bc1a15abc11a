"""The allocation-free compaction entry point against the workspace one, through the C ABI.

abm_select_indices_noalloc exists for callers that cannot allocate device memory when they
select agents (a fixed device-memory budget owned by a host application, or a loop that
must not risk the synchronisation of cudaMalloc/cudaFree).  It keeps its scratch in a
fixed array inside the library and shares it between calls, so this file checks two calls
in a row (the second must not see the first's leftovers) and the size limit.  The file is
named to be collected last.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_N = 1 << 26


def _with_workspace(lib_mod, mask):
    from jaxabm_gb300 import _dev
    n = mask.numel()
    idx = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    wsb = lib_mod.load().abm_select_workspace_bytes(n)
    ws = torch.empty(max(wsb, 16), dtype=torch.uint8, device="cuda")
    st = lib_mod.load().abm_select_indices(_dev.ptr(mask), n, _dev.ptr(idx), _dev.ptr(cnt),
                                           _dev.ptr(ws), ws.numel(), None)
    assert st == 0
    torch.cuda.synchronize()
    c = int(cnt.item())
    return idx[:c].cpu().numpy(), c


def _no_alloc(lib_mod, mask):
    from jaxabm_gb300 import _dev
    n = mask.numel()
    idx = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    st = lib_mod.load().abm_select_indices_noalloc(_dev.ptr(mask), n, _dev.ptr(idx),
                                                   _dev.ptr(cnt), None)
    assert st == 0
    torch.cuda.synchronize()
    c = int(cnt.item())
    return idx[:c].cpu().numpy(), c


@pytest.mark.parametrize("n", [1, 4095, 4097, 100_003, 1 << 20, MAX_N])
def test_no_alloc_matches_workspace_entry_point(cuda, n):
    from jaxabm_gb300 import _lib
    rs = np.random.RandomState(n % 1000)
    # two calls in a row with different densities: the shared scratch keeps the first
    # call's contents, and the second result must not depend on them
    for density in (0.7, 0.05):
        m = torch.from_numpy(rs.rand(n) < density).cuda().view(torch.uint8)
        ref_idx, ref_c = _with_workspace(_lib, m)
        got_idx, got_c = _no_alloc(_lib, m)
        assert got_c == ref_c
        assert np.array_equal(got_idx, ref_idx)


def test_no_alloc_empty_and_unaligned(cuda):
    from jaxabm_gb300 import _lib
    m = torch.zeros(0, dtype=torch.uint8, device="cuda")
    assert _no_alloc(_lib, m)[1] == 0
    full = torch.from_numpy(np.random.RandomState(3).rand(9001) < 0.3).cuda().view(torch.uint8)
    sub = full[5:]  # not 16-byte aligned
    assert np.array_equal(_no_alloc(_lib, sub)[0], _with_workspace(_lib, sub)[0])


def test_no_alloc_rejects_sizes_beyond_limit(cuda):
    from jaxabm_gb300 import _dev, _lib
    n = MAX_N + 1
    m = torch.zeros(n, dtype=torch.uint8, device="cuda")
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    cnt = torch.empty(1, dtype=torch.int64, device="cuda")
    st = _lib.load().abm_select_indices_noalloc(_dev.ptr(m), n, _dev.ptr(idx), _dev.ptr(cnt),
                                                None)
    assert st == _lib.ABM_ERR_BADARG
