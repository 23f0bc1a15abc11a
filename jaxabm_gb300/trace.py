"""NVTX ranges for profilers (Nsight Systems / Nsight Compute ``--nvtx``).

Off by default.  ``set_tracing(True)`` or ``JAXABM_NVTX=1`` in the environment opens a
range around every C-ABI call (named after the entry point, e.g. ``abm_sir_run``), every
``Model.run`` / ``Model.step`` and collection update, every batched replay and every
server tick, so a timeline shows which API call issued which kernels.  The ranges are
host-side markers on the calling thread; they add no synchronisation.
"""

import contextlib
import os

_ON = [os.environ.get("JAXABM_NVTX", "0") not in ("", "0")]


def set_tracing(flag: bool) -> None:
    _ON[0] = bool(flag)


def tracing() -> bool:
    return _ON[0]


def _nvtx():
    import torch
    return torch.cuda.nvtx


@contextlib.contextmanager
def nvtx_range(name: str):
    """``with nvtx_range("Model.run"):`` -- a push/pop pair when tracing is on (the pop
    also runs when the body raises), nothing otherwise."""
    if not _ON[0]:
        yield
        return
    nv = _nvtx()
    nv.range_push(name)
    try:
        yield
    finally:
        nv.range_pop()
