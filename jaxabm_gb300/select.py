"""Host side of K6 (stable compaction) and K7 (reductions) over SoA agent states.

``compact_states`` is ``AgentCollection.filter`` / ``AgentList.select``
(jaxabm/agent.py:213-243, jaxabm/agentpy.py:316-345): the mask is compacted into ascending
indices by the warp-ballot kernel, the count is read back once (the reference's
``int(jnp.sum(mask))`` host sync), and every attribute is gathered by row.
"""

import torch

from . import _dev
from . import _lib

REDUCE_SUM, REDUCE_MEAN, REDUCE_MIN, REDUCE_MAX = 0, 1, 2, 3


def _as_mask(mask, n):
    if not isinstance(mask, torch.Tensor):
        mask = torch.as_tensor(mask)
    if mask.device.type != "cuda":
        mask = mask.to(_dev.device())
    mask = mask.reshape(-1)
    if mask.numel() != n:
        raise ValueError(f"mask has {mask.numel()} entries for {n} agents")
    if mask.dtype == torch.bool:
        mask = mask.view(torch.uint8)
    elif mask.dtype != torch.uint8:
        mask = (mask != 0).view(torch.uint8)
    return mask.contiguous()


def select_indices(mask, n=None):
    """Ascending int32 indices of the true entries and their count (one host sync)."""
    if n is None:
        n = mask.numel()
    m = _as_mask(mask, n)
    idx = _dev.empty((max(n, 1),), torch.int32)
    count = _dev.empty((1,), torch.int64)
    ws = _dev.workspace(_lib.load().abm_select_workspace_bytes(n))
    _lib.call("abm_select_indices", _dev.ptr(m), n, _dev.ptr(idx), _dev.ptr(count), _dev.ptr(ws),
              ws.numel(), _dev.stream_handle())
    c = int(count.item())
    return idx[:c], c


def gather_rows(t, idx):
    """``t[idx]`` along dim 0 via the library's row gather."""
    t = t.contiguous()
    count = idx.numel()
    out = torch.empty((count,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    if count == 0:
        return out
    row_bytes = t.element_size() * (t[0].numel() if t.dim() > 1 else 1)
    _lib.call("abm_gather_rows", _dev.ptr(t), t.shape[0], row_bytes, _dev.ptr(idx), count,
              _dev.ptr(out), _dev.stream_handle())
    return out


def compact_states(states, mask):
    """(``{k: v[mask]}``, count) with ascending order preserved."""
    n = next(iter(states.values())).shape[0]
    idx, count = select_indices(mask, n)
    out = {}
    for k, v in states.items():
        if isinstance(v, torch.Tensor) and v.dim() >= 1 and v.shape[0] == n:
            out[k] = gather_rows(v, idx)
        else:
            out[k] = v
    return out, count


def reduce(x, op=REDUCE_MEAN):
    """Device float32 scalar: sum/mean/min/max of a float tensor (float64 accumulation)."""
    if not isinstance(x, torch.Tensor) or not x.is_cuda:
        raise ValueError("reduce expects a CUDA tensor")
    x32 = x.reshape(-1).to(torch.float32).contiguous()
    n = x32.numel()
    out = _dev.empty((), torch.float32)
    if n == 0:
        out.fill_(float("nan"))
        return out
    ws = _dev.workspace(_lib.load().abm_reduce_workspace_bytes(n))
    _lib.call("abm_reduce_f32", _dev.ptr(x32), n, int(op), _dev.ptr(out), _dev.ptr(ws),
              ws.numel(), _dev.stream_handle())
    return out


def mean(x):
    return reduce(x, REDUCE_MEAN)
