"""Oracle-side inputs of the workloads: networks, initial compartments and the 4,096-member
SIR ensemble.  TEST INFRASTRUCTURE ONLY (the checker and the CPU baseline build their inputs
here, without the shipped package).

* ``barabasi_albert`` / ``random_regular``: the C restatement in ``abm_oracle_graph.c``
  (CPU tests prove them equal to the library's generator and check the degree statistics
  that make a graph Barabasi-Albert or d-regular).
* ``sir_initial_states``: ``max(1, int(fraction * n))`` infected agents, the first entries
  of ``numpy.random.RandomState(seed).permutation(n)``.
* ``sir_ensemble_spec``: member sizes log-uniform in [1e3, 1e5] (``RandomState(seed)``),
  (beta, gamma) from a scrambled 2-D Sobol sequence seeded with ``seed`` scaled to
  [0.01, 0.2] x [0.05, 0.3], Poisson arrivals at 200 requests/s (``RandomState(seed + 1)``
  exponential gaps), model seed = member index.
"""

import ctypes
import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import build as _build


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def barabasi_albert(n, m=4, seed=0):
    """Symmetric CSR (row_ptr int32[n+1], col int32[2 m (n - m)])."""
    n, m = int(n), int(m)
    rp = np.empty(n + 1, np.int32)
    col = np.empty(2 * m * (n - m), np.int32)
    rc = _build.load().orc_graph_barabasi_albert(
        ctypes.c_int64(n), ctypes.c_int32(m), ctypes.c_uint64(int(seed) & (2**64 - 1)), _p(rp),
        _p(col), ctypes.c_int64(col.size))
    if rc != 0:
        raise ValueError(f"Barabasi-Albert generator failed for n={n}, m={m}")
    return rp, col


def random_regular(n, d=16, seed=0):
    n, d = int(n), int(d)
    rp = np.empty(n + 1, np.int32)
    col = np.empty(n * d, np.int32)
    rc = _build.load().orc_graph_random_regular(
        ctypes.c_int64(n), ctypes.c_int32(d), ctypes.c_uint64(int(seed) & (2**64 - 1)), _p(rp),
        _p(col), ctypes.c_int64(col.size))
    if rc != 0:
        raise ValueError(f"random regular generator failed for n={n}, d={d}")
    return rp, col


def sir_initial_states(n, fraction=0.001, seed=0):
    st = np.zeros(int(n), np.int8)
    st[np.random.RandomState(int(seed)).permutation(int(n))[:max(1, int(fraction * n))]] = 1
    return st


def sir_ensemble_spec(count=4096, n_lo=1_000, n_hi=100_000, seed=2, rate=200.0):
    from scipy.stats import qmc
    rs = np.random.RandomState(seed)
    sizes = np.rint(np.exp(rs.uniform(math.log(n_lo), math.log(n_hi), size=count)))
    try:
        sobol = qmc.Sobol(d=2, scramble=True, rng=np.random.default_rng(seed))
    except TypeError:  # SciPy before 1.15 names the argument `seed`
        sobol = qmc.Sobol(d=2, scramble=True, seed=seed)
    u = sobol.random(count)
    gaps = np.random.RandomState(seed + 1).exponential(1.0 / rate, size=count)
    return {"n": sizes.astype(np.int64),
            "beta": (0.01 + 0.19 * u[:, 0]).astype(np.float32),
            "gamma": (0.05 + 0.25 * u[:, 1]).astype(np.float32),
            "arrival_s": np.cumsum(gaps) - gaps[0],
            "seed": np.arange(count, dtype=np.int64)}


def sir_member(spec, i, m=4, fraction=0.001):
    """(row_ptr, col, initial compartments) of ensemble member ``i``: graph and infections
    seeded with the member's model seed."""
    n, s = int(spec["n"][i]), int(spec["seed"][i])
    rp, col = barabasi_albert(n, m, s)
    return rp, col, sir_initial_states(n, fraction, s)


def sir_members(spec, indices, workers=None):
    """Members ``indices`` built on host threads (the generator releases the GIL)."""
    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(lambda i: sir_member(spec, i), list(indices)))


def balanced_slices(sizes, parts):
    """Split member indices 0..len(sizes)-1 into ``parts`` contiguous runs of nearly equal
    total size (every member in exactly one run)."""
    sizes = np.asarray(sizes, dtype=np.float64)
    cum = np.concatenate([[0.0], np.cumsum(sizes)])
    cuts = np.searchsorted(cum, np.linspace(0.0, cum[-1], parts + 1)[1:-1], side="left")
    bounds = np.concatenate([[0], cuts, [len(sizes)]]).astype(np.int64)
    return [np.arange(bounds[k], bounds[k + 1]) for k in range(parts)]
