"""Host logic of the sensitivity analysis: the oracle's shuffle and Latin-hypercube
sampling (jaxabm/analysis.py:67-95), and the correlation indices
(jaxabm/analysis.py:167-203).  No GPU."""

import numpy as np
import pytest
import torch

from oracle import threefry as tf
from oracle.sampling import lhs_samples as lhs_oracle


@pytest.mark.parametrize("n", [0, 1, 2, 7, 1000, 2000])
def test_oracle_permutation_is_a_shuffle(n):
    p = tf.permutation(tf.PRNGKey(3), n)
    assert sorted(p.tolist()) == list(range(n))
    assert np.array_equal(p, tf.permutation(tf.PRNGKey(3), n))
    if n > 20:
        assert not np.array_equal(p, np.arange(n))
        assert not np.array_equal(p, tf.permutation(tf.PRNGKey(4), n))


def test_oracle_permutation_rounds():
    """One sort round below n = 1626 (3 ln n < ln(2**32 - 1)), two above; a second round
    re-sorts by fresh bits drawn from the advanced key."""
    assert int(np.ceil(3 * np.log(1625) / np.log(2**32 - 1))) == 1
    assert int(np.ceil(3 * np.log(1627) / np.log(2**32 - 1))) == 2
    key = tf.PRNGKey(9)
    k1, s1 = tf.split(key)
    one = np.argsort(tf.bits(s1, (2000,)), kind="stable")
    _, s2 = tf.split(k1)
    two = one[np.argsort(tf.bits(s2, (2000,)), kind="stable")]
    assert np.array_equal(tf.permutation(key, 2000), two)


def test_lhs_oracle_stratified():
    """Every parameter's column puts exactly one sample in each of the n strata."""
    n, ranges = 64, [(0.05, 0.2), (1.0, 3.0), (-1.0, 1.0)]
    s = lhs_oracle(42, n, ranges)
    assert s.shape == (n, 3)
    for i, (lo, hi) in enumerate(ranges):
        u = (s[:, i].astype(np.float64) - lo) / (hi - lo)
        assert np.all(s[:, i] >= lo) and np.all(s[:, i] <= hi)
        strata = np.floor(u * n + 1e-4).astype(int)
        assert sorted(np.clip(strata, 0, n - 1).tolist()) == list(range(n))


def _bare(samples, results, ranges):
    from jaxabm_gb300.analysis import SensitivityAnalysis
    sa = SensitivityAnalysis.__new__(SensitivityAnalysis)
    sa.param_ranges = ranges
    sa.samples = torch.as_tensor(samples, dtype=torch.float32)
    sa.results = None if results is None else {k: torch.as_tensor(v, dtype=torch.float32)
                                                for k, v in results.items()}
    return sa


def test_sobol_indices_squared_correlation():
    rng = np.random.RandomState(0)
    s = rng.rand(50, 2).astype(np.float32)
    noise = rng.rand(50).astype(np.float32)
    res = {"lin": 3 * s[:, 0] + 1, "mix": s[:, 1] + 0.5 * noise}
    idx = _bare(s, res, {"a": (0, 1), "b": (0, 1)}).sobol_indices()
    assert idx["lin"]["a"] == pytest.approx(1.0, abs=1e-5)
    assert idx["lin"]["b"] < 0.2
    for m, v in res.items():
        for j, name in enumerate(("a", "b")):
            x = s[:, j]
            want = np.mean(((x - x.mean()) / (x.std() + 1e-8)) *
                           ((v - v.mean()) / (v.std() + 1e-8))) ** 2
            assert idx[m][name] == pytest.approx(float(want), rel=1e-4)
            assert isinstance(idx[m][name], float)


def test_sobol_indices_before_run_raises():
    with pytest.raises(ValueError):
        _bare(np.zeros((3, 1)), None, {"a": (0, 1)}).sobol_indices()
