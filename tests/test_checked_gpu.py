"""The range-checked build (``-DABM_CHECKED``, libjaxabm_gb300_checked.so).

On valid inputs it computes exactly what the normal build computes; an index outside its
array -- a CSR column >= n, a row offset past the last slot, a gather row >= the source's
row count -- comes back as ABM_ERR_BOUNDS with the entry point, index and bound in
``abm_bounds_detail()``, and the kernel keeps every access inside its arrays (the bad
index is redirected to element 0).  Bad inputs are given to the checked build only."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

B = 8


@pytest.fixture(scope="module")
def libs(lib):
    import jaxabm_gb300 as jx
    from jaxabm_gb300 import _lib
    checked = _lib.load(path=jx.build(checked=True))
    assert checked.abm_checked_build() == 1 and lib.abm_checked_build() == 0
    return lib, checked


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _ring(n):
    """Symmetric ring: node i has neighbours i-1 and i+1."""
    rp = np.arange(0, 2 * n + 1, 2, dtype=np.int32)
    col = np.empty(2 * n, dtype=np.int32)
    col[0::2] = (np.arange(n) - 1) % n
    col[1::2] = (np.arange(n) + 1) % n
    return rp, col


def _opinion_step(L, rp, col, n, seed=0):
    g = torch.Generator().manual_seed(seed)
    o = torch.rand((n, B), generator=g).cuda()
    out = torch.zeros_like(o)
    mu = torch.full((B,), 0.3, device="cuda")
    eps = torch.full((B,), 0.2, device="cuda")
    tau = torch.full((B,), 0.02, device="cuda")
    d_rp = torch.from_numpy(rp).cuda()
    d_col = torch.from_numpy(col).cuda()
    st = L.abm_opinion_step(_ptr(o), _ptr(out), _ptr(d_rp), _ptr(d_col), n, B, _ptr(mu),
                            _ptr(eps), _ptr(tau), None)
    torch.cuda.synchronize()
    return st, out.cpu()


def test_checked_equals_normal_on_valid_inputs(cuda, libs):
    lib, checked = libs
    n = 1000
    rp, col = _ring(n)
    s0, a = _opinion_step(lib, rp, col, n)
    s1, b = _opinion_step(checked, rp, col, n)
    assert s0 == 0 and s1 == 0
    assert torch.equal(a, b)
    src = torch.arange(40 * 3, dtype=torch.int32, device="cuda").view(40, 3)
    idx = torch.tensor([39, 0, 7, 7], dtype=torch.int32, device="cuda")
    outs = []
    for L in (lib, checked):
        out = torch.empty((4, 3), dtype=torch.int32, device="cuda")
        assert L.abm_gather_rows(_ptr(src), 40, 12, _ptr(idx), 4, _ptr(out), None) == 0
        torch.cuda.synchronize()
        outs.append(out.cpu())
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], src.cpu()[idx.cpu().long()])


def test_checked_reports_column_out_of_range(cuda, libs):
    _, checked = libs
    n = 500
    rp, col = _ring(n)
    col[301] = n  # one column one past the last node
    st, _ = _opinion_step(checked, rp, col, n)
    assert st == 4  # ABM_ERR_BOUNDS
    detail = checked.abm_bounds_detail().decode()
    assert "abm_opinion_step" in detail and f"index {n} outside [0, {n})" in detail
    # the status word is cleared: the next valid call is clean
    rp, col = _ring(n)
    assert _opinion_step(checked, rp, col, n)[0] == 0


def test_checked_reports_row_offsets_past_the_last_slot(cuda, libs):
    _, checked = libs
    n = 64
    rp, col = _ring(n)
    rp[10] = 2 * n + 5  # row 9 ends past rp[n]; row 10 starts there
    st, _ = _opinion_step(checked, rp, col, n)
    assert st == 4
    assert f"outside [0, {2 * n})" in checked.abm_bounds_detail().decode()


def test_checked_reports_gather_row_out_of_range(cuda, libs):
    _, checked = libs
    src = torch.zeros((10, 4), dtype=torch.float32, device="cuda")
    idx = torch.tensor([3, 10, 1], dtype=torch.int32, device="cuda")
    out = torch.empty((3, 4), dtype=torch.float32, device="cuda")
    st = checked.abm_gather_rows(_ptr(src), 10, 16, _ptr(idx), 3, _ptr(out), None)
    assert st == 4
    assert "abm_gather_rows: index 10 outside [0, 10)" in checked.abm_bounds_detail().decode()


def test_python_error_carries_the_detail(cuda, libs, monkeypatch):
    from jaxabm_gb300 import _lib
    _, checked = libs
    monkeypatch.setattr(_lib, "_lib", checked)
    src = torch.zeros((5, 2), dtype=torch.int32, device="cuda")
    idx = torch.tensor([-1], dtype=torch.int32, device="cuda")
    out = torch.empty((1, 2), dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.AbmError, match=r"index out of bounds.*index -1 outside \[0, 5\)"):
        _lib.call("abm_gather_rows", _ptr(src), 5, 8, _ptr(idx), 1, _ptr(out), None)
