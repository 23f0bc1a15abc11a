"""Small helpers shared by the host-side wrappers: device checks, raw pointers, streams."""

import numpy as np
import torch


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("jaxabm_gb300 runs on a CUDA device; none is available")


def device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def ptr(t, name="tensor"):
    """Raw device pointer of a contiguous CUDA tensor (borrowed for one C-ABI call)."""
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must live on a CUDA device")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return t.data_ptr()


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def empty(shape, dtype):
    return torch.empty(shape, dtype=dtype, device=device())


def workspace(nbytes):
    """Caller-side workspace for an entry point (the library never allocates)."""
    n = max(int(nbytes), 16)
    return torch.empty(n, dtype=torch.uint8, device=device())


def keys_to_numpy(t):
    """int32-stored key tensor -> numpy uint32 (same bits)."""
    return t.detach().cpu().numpy().astype(np.int32).view(np.uint32)


def keys_from_numpy(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.uint32))
    return torch.from_numpy(a.view(np.int32).copy()).to(device())
