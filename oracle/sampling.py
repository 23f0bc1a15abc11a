"""CPU oracle for the sensitivity analysis's Latin-hypercube sampling.

TEST INFRASTRUCTURE ONLY: used by ``tests/`` as the checker, never by the package.

Restates ``SensitivityAnalysis._generate_lhs_samples`` (jaxabm/analysis.py:67-95) on the
oracle's ``jax.random`` (``threefry.py``): ``key, sub = split(PRNGKey(seed))``; stratum
starts ``linspace(0, 1, n + 1)[:-1]`` (= ``i / n`` in float32); plus
``uniform(sub, (n,)) / n``; per parameter ``key, sub = split(key)`` and
``permutation(sub, points)``; then ``* (max - min) + min`` in float32.  Parity unpinned
against JAX itself (not installed), like the rest of the oracle's samplers.
"""

import numpy as np

from . import threefry as tf


def lhs_samples(seed, n, ranges):
    """float32 ``(n, len(ranges))`` samples for ``ranges`` = [(min, max), ...]."""
    key = tf.PRNGKey(seed)
    key, sub = tf.split(key)
    points = np.arange(n, dtype=np.float32) / np.float32(n)
    points = points + tf.uniform(sub, (n,)).astype(np.float32) / np.float32(n)
    cols = []
    for _ in ranges:
        key, sub = tf.split(key)
        cols.append(tf.permutation(sub, points))
    out = (np.stack(cols, axis=1) if cols else np.zeros((n, 0))).astype(np.float32)
    for i, (lo, hi) in enumerate(ranges):
        out[:, i] *= np.float32(hi - lo)
        out[:, i] += np.float32(lo)
    return out
