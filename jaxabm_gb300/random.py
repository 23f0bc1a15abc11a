"""Device-side ``jax.random`` for the engine: threefry2x32 keys and samplers on CUDA.

Keys are int32 tensors of shape ``(..., 2)`` on the GPU holding the same 64 bits as a JAX
raw ``uint32[2]`` key (``PRNGKey(seed)`` = ``[seed >> 32, seed & 0xffffffff]``).  Leading
dimensions behave like ``jax.vmap`` over keys.  All sampling runs in the CUDA library
(K1 kernels); see ``jax.random`` as called from jaxabm/model.py:46,129,156,164,183 and
jaxabm/agent.py:115,156.

``jax_threefry_partitionable`` (True by default since JAX 0.5.0) is mirrored by
:func:`set_partitionable`; the model kernels always use the partitionable mode.
"""

import math

import numpy as np
import torch

from . import _dev
from . import _lib

_MODE = [_lib.RNG_PARTITIONABLE]


def set_partitionable(flag: bool) -> None:
    """Select ``jax_threefry_partitionable`` semantics for the samplers in this module."""
    _MODE[0] = _lib.RNG_PARTITIONABLE if flag else _lib.RNG_LEGACY


def partitionable() -> bool:
    return _MODE[0] == _lib.RNG_PARTITIONABLE


def PRNGKey(seed: int) -> torch.Tensor:
    """``jax.random.PRNGKey(seed)`` as a device int32[2] tensor."""
    seed = int(seed)
    hi, lo = (seed >> 32) & 0xFFFFFFFF, seed & 0xFFFFFFFF
    return _dev.keys_from_numpy(np.array([hi, lo], dtype=np.uint32))


def key_data(key: torch.Tensor) -> np.ndarray:
    """Host uint32 copy of a key array (``jax.random.key_data``)."""
    return _dev.keys_to_numpy(key)


def _flat_keys(key):
    if key.dtype != torch.int32 or key.shape[-1] != 2:
        raise TypeError("a key is an int32 tensor with a trailing dimension of 2")
    lead = tuple(key.shape[:-1])
    return key.contiguous().reshape(-1, 2), lead


def _shape(shape):
    if isinstance(shape, int):
        shape = (shape,)
    shape = tuple(int(s) for s in shape)
    return shape, int(math.prod(shape)) if shape else 1


def split(key: torch.Tensor, num: int = 2) -> torch.Tensor:
    """``jax.random.split(key, num)`` -> int32[..., num, 2]."""
    flat, lead = _flat_keys(key)
    out = _dev.empty((flat.shape[0], int(num), 2), torch.int32)
    _lib.call("abm_rng_split", _dev.ptr(flat), flat.shape[0], int(num), _dev.ptr(out), _MODE[0],
              _dev.stream_handle())
    return out.reshape(*lead, int(num), 2)


def bits(key: torch.Tensor, shape=()) -> torch.Tensor:
    """``jax.random.bits(key, shape)`` (32-bit words, stored as int32)."""
    flat, lead = _flat_keys(key)
    shape, count = _shape(shape)
    out = _dev.empty((flat.shape[0], count), torch.int32)
    _lib.call("abm_rng_bits", _dev.ptr(flat), flat.shape[0], count, _dev.ptr(out), _MODE[0],
              _dev.stream_handle())
    return out.reshape(lead + shape)


def uniform(key: torch.Tensor, shape=(), minval=0.0, maxval=1.0) -> torch.Tensor:
    """``jax.random.uniform(key, shape, float32, minval, maxval)``."""
    flat, lead = _flat_keys(key)
    shape, count = _shape(shape)
    out = _dev.empty((flat.shape[0], count), torch.float32)
    _lib.call("abm_rng_uniform", _dev.ptr(flat), flat.shape[0], count, float(minval),
              float(maxval), _dev.ptr(out), _MODE[0], _dev.stream_handle())
    return out.reshape(lead + shape)


def normal(key: torch.Tensor, shape=()) -> torch.Tensor:
    """``jax.random.normal(key, shape, float32)``."""
    flat, lead = _flat_keys(key)
    shape, count = _shape(shape)
    out = _dev.empty((flat.shape[0], count), torch.float32)
    _lib.call("abm_rng_normal", _dev.ptr(flat), flat.shape[0], count, _dev.ptr(out), _MODE[0],
              _dev.stream_handle())
    return out.reshape(lead + shape)


def bernoulli(key: torch.Tensor, p=0.5, shape=()) -> torch.Tensor:
    """``jax.random.bernoulli(key, p, shape)`` -> bool tensor."""
    flat, lead = _flat_keys(key)
    shape, count = _shape(shape)
    out = _dev.empty((flat.shape[0], count), torch.uint8)
    _lib.call("abm_rng_bernoulli", _dev.ptr(flat), flat.shape[0], count, float(p), _dev.ptr(out),
              _MODE[0], _dev.stream_handle())
    return out.reshape(lead + shape).bool()


def randint(key: torch.Tensor, shape, minval, maxval) -> torch.Tensor:
    """``jax.random.randint(key, shape, minval, maxval, int32)``."""
    flat, lead = _flat_keys(key)
    shape, count = _shape(shape)
    out = _dev.empty((flat.shape[0], count), torch.int32)
    _lib.call("abm_rng_randint", _dev.ptr(flat), flat.shape[0], count, int(minval), int(maxval),
              _dev.ptr(out), _MODE[0], _dev.stream_handle())
    return out.reshape(lead + shape)


def permutation(key: torch.Tensor, x) -> torch.Tensor:
    """``jax.random.permutation(key, x)`` for an int ``x`` (a shuffle of ``arange(x)``) or a
    1-D tensor (its entries shuffled, on the device).  JAX's shuffle: ``ceil(3 ln n /
    ln(2**32 - 1))`` rounds, each splitting the key into (key, subkey) and stably sorting
    the entries by ``bits(subkey, (n,))`` read as unsigned words."""
    if isinstance(x, int):
        arr = torch.arange(int(x), device=_dev.device())
    else:
        arr = torch.as_tensor(x).to(_dev.device())
        if arr.dim() != 1:
            raise ValueError("permutation takes an int or a 1-D tensor")
    n = arr.shape[0]
    rounds = int(math.ceil(3 * math.log(max(1, n)) / math.log(2.0**32 - 1)))
    for _ in range(rounds):
        pair = split(key, 2)
        key, sub = pair[0], pair[1]
        words = bits(sub, (n,)).to(torch.int64) & 0xFFFFFFFF
        arr = arr[torch.sort(words, stable=True).indices]
    return arr


def keychain(rng: torch.Tensor, steps: int, ncoll: int = 1, update_keys: bool = False):
    """Advance ``rng`` (int32[..., 2], in place) through ``steps`` calls of Model.step and
    return the per-step collection keys int32[..., steps, ncoll, 2]
    (jaxabm/model.py:155-168); with ``update_keys`` also the update_state_fn keys
    int32[..., steps, 2] (jaxabm/model.py:182-183)."""
    if not rng.is_contiguous():
        raise ValueError("rng must be contiguous (it is advanced in place)")
    flat, lead = _flat_keys(rng)
    out = _dev.empty((flat.shape[0], int(steps), int(ncoll), 2), torch.int32)
    upd = _dev.empty((flat.shape[0], int(steps), 2), torch.int32) if update_keys else None
    _lib.call("abm_keychain", _dev.ptr(flat), flat.shape[0], int(ncoll), int(steps),
              _dev.ptr(out), _dev.ptr(upd) if upd is not None else None, _dev.stream_handle())
    out = out.reshape(*lead, int(steps), int(ncoll), 2)
    if update_keys:
        return out, upd.reshape(*lead, int(steps), 2)
    return out
