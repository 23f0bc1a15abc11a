"""CPU oracle for the ``jax.random`` key and sampling semantics (NumPy, uint32).

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped package imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it,
and only as the checker.

Parity status: UNPINNED against the reference.  The reference (JaxABM 0.1.5) reaches its
random numbers through the third-party package ``jax`` (``requirements.txt``: ``jax>=0.4.1``,
no lock file), which is not installed here and ships no known-answer vectors of its own
path.  This module restates the published algorithms instead:

* Threefry-2x32 with 20 rounds, Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
  easy as 1, 2, 3", SC'11 (Random123).  Rotation schedule 13,15,26,6 / 17,29,16,24, key
  parity constant 0x1BD11BDA, key injection after every fourth round.
* ``jax.random`` (JAX >= 0.5.0, where ``jax_threefry_partitionable`` defaults to True; the
  pre-0.5 "original" mode is provided as ``mode=LEGACY``):

  - ``PRNGKey(seed)``  -> ``[seed >> 32, seed & 0xffffffff]`` (uint32 pair)
  - ``split(key, n)``  -> partitionable: key i = threefry(key, (hi(i), lo(i)));
                          legacy: threefry over iota(2n) with the first half of the
                          counters paired with the second half, reshaped to (n, 2)
  - ``bits(key, shape)``  partitionable: word i = y0 ^ y1 of threefry(key, (hi(i), lo(i)));
                          legacy: threefry over iota(size), half-paired, zero-padded
  - ``uniform``  top 23 bits as the mantissa of a float in [1, 2), minus 1, scaled,
                 shifted and clamped below at minval
  - ``normal``   sqrt(2) * erfinv(uniform(nextafter(-1, 0), 1))
  - ``bernoulli``  uniform(key, shape) < p

The reference's own call sites are ``jaxabm/model.py:46,129,156,164,183`` and
``jaxabm/agent.py:115,156`` (key chain) and ``jaxabm/agentpy.py:509-512`` (Grid placement).
"""

import numpy as np

PARTITIONABLE = 1
LEGACY = 0

_ROT = (13, 15, 26, 6, 17, 29, 16, 24)
_PARITY = np.uint32(0x1BD11BDA)


def _rotl(x, r):
    r = np.uint32(r)
    return (x << r) | (x >> np.uint32(32 - int(r)))


def threefry2x32(k0, k1, x0, x1):
    """Threefry-2x32-20 block function, elementwise over broadcastable uint32 arrays.

    Follows the Random123 specification (Salmon et al., SC'11, table of rotation
    constants for 2x32 and the Skein key schedule).
    """
    with np.errstate(over="ignore"):
        k0 = np.asarray(k0, dtype=np.uint32)
        k1 = np.asarray(k1, dtype=np.uint32)
        x0 = np.array(x0, dtype=np.uint32, copy=True)
        x1 = np.array(x1, dtype=np.uint32, copy=True)
        x0, x1, k0, k1 = np.broadcast_arrays(x0, x1, k0, k1)
        x0 = x0.copy()
        x1 = x1.copy()
        ks = (k0, k1, k0 ^ k1 ^ _PARITY)
        x0 += ks[0]
        x1 += ks[1]
        for s in range(5):
            base = 0 if s % 2 == 0 else 4
            for r in range(4):
                x0 += x1
                x1 = _rotl(x1, _ROT[base + r])
                x1 ^= x0
            x0 += ks[(s + 1) % 3]
            x1 += ks[(s + 2) % 3] + np.uint32(s + 1)
        return x0, x1


def PRNGKey(seed):
    """``jax.random.PRNGKey``: uint32[2] = (seed >> 32, seed & 0xffffffff)."""
    seed = int(seed)
    return np.array([(seed >> 32) & 0xFFFFFFFF, seed & 0xFFFFFFFF], dtype=np.uint32)


def _iota_hi_lo(n):
    i = np.arange(n, dtype=np.uint64)
    return (i >> np.uint64(32)).astype(np.uint32), (i & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def _threefry_halves(key, count):
    """JAX's ``threefry_2x32(keypair, count)``: first half of the flattened counter array
    is paired with the second half (zero-padded to even length), outputs concatenated."""
    count = np.asarray(count, dtype=np.uint32).ravel()
    n = count.size
    if n % 2:
        count = np.concatenate([count, np.zeros(1, np.uint32)])
    h = count.size // 2
    y0, y1 = threefry2x32(key[0], key[1], count[:h], count[h:])
    out = np.concatenate([y0, y1])
    return out[:n]


def split(key, num=2, mode=PARTITIONABLE):
    """``jax.random.split(key, num)`` -> uint32[num, 2]."""
    key = np.asarray(key, dtype=np.uint32)
    if mode == PARTITIONABLE:
        hi, lo = _iota_hi_lo(num)
        y0, y1 = threefry2x32(key[0], key[1], hi, lo)
        return np.stack([y0, y1], axis=-1)
    out = _threefry_halves(key, np.arange(2 * num, dtype=np.uint32))
    return out.reshape(num, 2)


def split_batched(keys, num, mode=PARTITIONABLE):
    """``vmap(lambda k: split(k, num))(keys)`` -> uint32[nkeys, num, 2]."""
    keys = np.asarray(keys, dtype=np.uint32).reshape(-1, 2)
    if mode == PARTITIONABLE:
        hi, lo = _iota_hi_lo(num)
        y0, y1 = threefry2x32(keys[:, :1], keys[:, 1:], hi[None, :], lo[None, :])
        return np.stack([y0, y1], axis=-1)
    return np.stack([split(k, num, mode) for k in keys])


def bits(key, shape=(), mode=PARTITIONABLE):
    """``jax.random.bits(key, shape)`` for 32-bit words -> uint32[shape]."""
    key = np.asarray(key, dtype=np.uint32)
    size = int(np.prod(shape)) if len(shape) else 1
    if mode == PARTITIONABLE:
        hi, lo = _iota_hi_lo(size)
        y0, y1 = threefry2x32(key[0], key[1], hi, lo)
        out = y0 ^ y1
    else:
        out = _threefry_halves(key, np.arange(size, dtype=np.uint32))
    return out.reshape(shape)


def bits_batched(keys, count, mode=PARTITIONABLE):
    """``vmap(lambda k: bits(k, (count,)))(keys)`` -> uint32[nkeys, count]."""
    keys = np.asarray(keys, dtype=np.uint32).reshape(-1, 2)
    if mode == PARTITIONABLE:
        hi, lo = _iota_hi_lo(count)
        y0, y1 = threefry2x32(keys[:, :1], keys[:, 1:], hi[None, :], lo[None, :])
        return y0 ^ y1
    return np.stack([bits(k, (count,), mode) for k in keys])


def bits_to_unit_float(b):
    """Top 23 bits -> float32 in [0, 1): exactly k * 2**-23 with k = b >> 9."""
    b = np.asarray(b, dtype=np.uint32)
    f = ((b >> np.uint32(9)) | np.uint32(0x3F800000)).view(np.float32)
    return (f - np.float32(1.0)).astype(np.float32)


def uniform_from_bits(b, minval=0.0, maxval=1.0):
    minval = np.float32(minval)
    maxval = np.float32(maxval)
    u = bits_to_unit_float(b)
    span = np.float32(maxval - minval)
    # one multiply and one add, each rounded to float32 (no fused multiply-add)
    v = (u * span).astype(np.float32)
    v = (v + minval).astype(np.float32)
    return np.maximum(minval, v).astype(np.float32)


def uniform(key, shape=(), minval=0.0, maxval=1.0, mode=PARTITIONABLE):
    """``jax.random.uniform(key, shape, float32, minval, maxval)``."""
    return uniform_from_bits(bits(key, shape, mode), minval, maxval)


NORMAL_LO = np.nextafter(np.float32(-1.0), np.float32(0.0), dtype=np.float32)

# Giles, "Approximating the erfinv function", GPU Computing Gems Jade (2011): the
# single-precision central (w < 5) and tail (w >= 5) polynomials, highest degree first.
GILES_CENTRAL = (2.81022636e-08, 3.43273939e-07, -3.5233877e-06, -4.39150654e-06,
                 0.00021858087, -0.00125372503, -0.00417768164, 0.246640727, 1.50140941)
GILES_TAIL = (-0.000200214257, 0.000100950558, 0.00134934322, -0.00367342844,
              0.00573950773, -0.0076224613, 0.00943887047, 1.00167406, 2.83297682)


def erfinv_f64(x):
    """Inverse error function in float64 (Newton-refined), the FP64 reference value."""
    from scipy.special import erfinv
    return erfinv(np.asarray(x, dtype=np.float64))


def erfinv_giles_f32(x):
    """Giles' single-precision erfinv, evaluated in float32 with w = -log1p(-x*x) and a
    fused multiply-add Horner scheme (the product of two float32 values is exact in
    float64, so one rounding of p*w + c to float32 models fmaf)."""
    x = np.asarray(x, dtype=np.float32)
    w = -np.log1p(-(x * x).astype(np.float32)).astype(np.float32)
    central = w < np.float32(5.0)
    wc = np.where(central, w - np.float32(2.5), np.sqrt(w) - np.float32(3.0)).astype(np.float32)
    p = np.where(central, np.float32(GILES_CENTRAL[0]), np.float32(GILES_TAIL[0])).astype(np.float32)
    for a, b in zip(GILES_CENTRAL[1:], GILES_TAIL[1:]):
        c = np.where(central, np.float32(a), np.float32(b)).astype(np.float32)
        p = (p.astype(np.float64) * wc.astype(np.float64) + c.astype(np.float64)).astype(np.float32)
    return (p * x).astype(np.float32)


SQRT2_F32 = np.float32(np.sqrt(2.0))


def normal_from_bits(b):
    u = uniform_from_bits(b, NORMAL_LO, 1.0)
    return (SQRT2_F32 * erfinv_giles_f32(u)).astype(np.float32)


def normal_from_bits_f64(b):
    """Same draw with the inverse error function taken in float64 (FP64 reference)."""
    u = uniform_from_bits(b, NORMAL_LO, 1.0).astype(np.float64)
    return np.sqrt(2.0) * erfinv_f64(u)


def normal(key, shape=(), mode=PARTITIONABLE):
    """``jax.random.normal(key, shape, float32)``."""
    return normal_from_bits(bits(key, shape, mode))


def bernoulli(key, p=0.5, shape=(), mode=PARTITIONABLE):
    """``jax.random.bernoulli(key, p, shape)`` = uniform(key, shape) < float32(p)."""
    return uniform(key, shape, mode=mode) < np.float32(p)


def randint(key, shape, minval, maxval, mode=PARTITIONABLE):
    """``jax.random.randint(key, shape, minval, maxval, int32)``: two bit draws from
    ``split(key)`` combined modulo the span in wrapping uint32 arithmetic."""
    k = split(key, 2, mode)
    hi = bits(k[0], shape, mode).astype(np.uint64)
    lo = bits(k[1], shape, mode).astype(np.uint64)
    span = 1 if maxval <= minval else (int(maxval) - int(minval)) & 0xFFFFFFFF
    mult = 65536 % span
    mult = ((mult * mult) & 0xFFFFFFFF) % span  # the square wraps in uint32, as in JAX
    r = (((hi % span) * np.uint64(mult)) & np.uint64(0xFFFFFFFF)) + (lo % span)
    r = (r & np.uint64(0xFFFFFFFF)) % np.uint64(span)
    return ((np.int64(minval) + r.astype(np.int64)) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)


def permutation(key, x, mode=PARTITIONABLE):
    """``jax.random.permutation(key, x)`` for an int ``x`` (a shuffle of ``arange(x)``) or a
    1-D array (its entries shuffled).  Published JAX shuffle (``jax/_src/random.py``,
    ``_shuffle``): ``ceil(3 ln n / ln(2**32 - 1))`` rounds; each round splits the key into
    (key, subkey) and stably sorts the entries by ``bits(subkey, (n,))``."""
    arr = np.arange(int(x)) if np.ndim(x) == 0 else np.asarray(x).copy()
    n = arr.shape[0]
    rounds = int(np.ceil(3 * np.log(max(1, n)) / np.log(np.iinfo(np.uint32).max)))
    key = np.asarray(key, dtype=np.uint32)
    for _ in range(rounds):
        key, sub = split(key, 2, mode)
        order = np.argsort(bits(sub, (n,), mode), kind="stable")
        arr = arr[order]
    return arr
