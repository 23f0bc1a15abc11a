"""abm_copy_segments_kernel: many host<->device copies in one launch, equal byte for byte to
the per-segment copies, at every alignment; pageable or unknown pointers are refused on the
host (ABM_ERR_BADARG) before anything is launched."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _table(rows):
    t = torch.empty((len(rows), 3), dtype=torch.int64, pin_memory=True)
    v = t.numpy().view(np.uint64)
    for k, (d, s, n) in enumerate(rows):
        v[k] = (d, s, n)
    return t


def test_gather_copies_match_at_every_alignment(cuda, lib):
    rng = np.random.default_rng(0)
    host = torch.from_numpy(rng.integers(0, 256, 1 << 20, dtype=np.uint8)).pin_memory()
    dev = torch.zeros(1 << 20, dtype=torch.uint8, device="cuda")
    # (dst offset, src offset, bytes): equal alignment mod 16, mod 4 only, none, empty,
    # shorter than one vector, long
    segs = [(0, 0, 100_000), (200_003, 300_003, 70_001), (400_001, 500_002, 5_555),
            (600_002, 600_010, 9_999), (700_000, 700_000, 0), (710_005, 720_005, 7),
            (800_000, 16, 200_000)]
    rows = [(dev.data_ptr() + d, host.data_ptr() + s, n) for d, s, n in segs]
    table = _table(rows)
    st = lib.abm_copy_segments_kernel(ctypes.c_void_p(table.data_ptr()), len(rows), None)
    assert st == 0
    torch.cuda.synchronize()
    got, want = dev.cpu().numpy(), np.zeros(1 << 20, dtype=np.uint8)
    h = host.numpy()
    for d, s, n in segs:
        want[d:d + n] = h[s:s + n]
    assert np.array_equal(got, want)
    # device -> page-locked host, the other direction of the same launch
    back = torch.zeros(1 << 20, dtype=torch.uint8).pin_memory()
    rows = [(back.data_ptr() + s, dev.data_ptr() + d, n) for d, s, n in segs]
    table = _table(rows)
    assert lib.abm_copy_segments_kernel(ctypes.c_void_p(table.data_ptr()), len(rows), None) == 0
    torch.cuda.synchronize()
    b = back.numpy()
    for d, s, n in segs:
        assert np.array_equal(b[s:s + n], got[d:d + n])


def test_gather_copy_refuses_pageable_memory(cuda, lib):
    dev = torch.zeros(64, dtype=torch.uint8, device="cuda")
    pageable = np.arange(64, dtype=np.uint8)
    table = _table([(dev.data_ptr(), pageable.ctypes.data, 64)])
    assert lib.abm_copy_segments_kernel(ctypes.c_void_p(table.data_ptr()), 1, None) == 1
    # the table itself must be device-accessible too
    plain = np.array([[dev.data_ptr(), dev.data_ptr(), 0]], dtype=np.uint64)
    assert lib.abm_copy_segments_kernel(ctypes.c_void_p(plain.ctypes.data), 1, None) == 1
    assert lib.abm_copy_segments_kernel(None, 1, None) == 1
    assert lib.abm_copy_segments_kernel(None, 0, None) == 0
    torch.cuda.synchronize()
    assert not dev.any()
