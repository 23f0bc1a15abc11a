"""Sensitivity analysis on the ensemble engine (jaxabm/analysis.py:23-203): device
``permutation`` and Latin-hypercube samples against the oracle, a batched SIR analysis
against each sample's model run alone, and the serial path for other models."""

import numpy as np
import pytest
import torch

from oracle import threefry as tf
from oracle.sampling import lhs_samples as lhs_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 5, 100, 2000])
def test_permutation_matches_oracle(cuda, n):
    from jaxabm_gb300 import random as jr
    got = jr.permutation(jr.PRNGKey(11), n).cpu().numpy()
    assert np.array_equal(got, tf.permutation(tf.PRNGKey(11), n))
    x = torch.linspace(0, 1, n, device=cuda)
    got = jr.permutation(jr.PRNGKey(12), x).cpu().numpy()
    assert np.array_equal(got, tf.permutation(tf.PRNGKey(12), x.cpu().numpy()))


def test_lhs_samples_match_oracle(cuda):
    import jaxabm_gb300 as jx
    ranges = {"beta": (0.02, 0.2), "gamma": (0.05, 0.3), "other": (-1.0, 4.0)}
    sa = jx.SensitivityAnalysis(lambda params, config: None, ranges, ["I"], num_samples=37,
                                seed=42)
    want = lhs_oracle(42, 37, list(ranges.values()))
    assert sa.samples.shape == (37, 3) and sa.samples.dtype == torch.float32
    assert np.array_equal(sa.samples.cpu().numpy(), want)


def test_sir_analysis_runs_batched_and_matches_serial(cuda):
    import jaxabm_gb300 as jx

    def factory(params=None, config=None):
        p = {"n": 2500, "m": 3, "steps": 40, "initial_infected": 0.01}
        p.update(params or {})
        return jx.SIRModel(p, seed=config.seed)

    sa = jx.SensitivityAnalysis(factory, {"beta": (0.02, 0.3), "gamma": (0.05, 0.4)},
                                ["I", "R", "S"], num_samples=6, seed=3)
    res = sa.run(verbose=False)
    assert sa.batched
    host = sa.samples.cpu().numpy()
    for i in range(6):
        params = {"beta": float(host[i, 0]), "gamma": float(host[i, 1])}
        ref = factory(params=params, config=jx.ModelConfig(seed=1000 + i)).run()
        for m in ("I", "R", "S"):
            assert res[m].shape == (6,)
            assert float(res[m][i]) == float(ref[m][-1]), (i, m)
    idx = sa.sobol_indices()
    assert set(idx) == {"I", "R", "S"} and set(idx["R"]) == {"beta", "gamma"}


def test_non_sir_analysis_runs_serially(cuda):
    import jaxabm_gb300 as jx

    def factory(params=None, config=None):
        p = {"n": 500, "steps": 5}
        p.update(params or {})
        return jx.RandomWalkModel(p, seed=config.seed)

    sa = jx.SensitivityAnalysis(factory, {"sigma": (0.001, 0.05)}, ["mean_x", "missing"],
                                num_samples=3, seed=1)
    res = sa.run(verbose=False)
    assert not sa.batched
    for i in range(3):
        ref = factory(params={"sigma": float(sa.samples[i, 0])},
                      config=jx.ModelConfig(seed=1000 + i)).run()
        assert float(res["mean_x"][i]) == pytest.approx(float(ref["mean_x"][-1]), rel=1e-6)
    assert torch.all(res["missing"] == 0)
