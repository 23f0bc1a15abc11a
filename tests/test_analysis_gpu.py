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


def test_random_walk_analysis_is_batched(cuda):
    import jaxabm_gb300 as jx

    def factory(params=None, config=None):
        p = {"n": 500, "steps": 5}
        p.update(params or {})
        return jx.RandomWalkModel(p, seed=config.seed)

    sa = jx.SensitivityAnalysis(factory, {"sigma": (0.001, 0.05)}, ["mean_x", "missing"],
                                num_samples=3, seed=1)
    res = sa.run(verbose=False)
    assert sa.batched  # random-walk samples run as one batch, each equal to its own run()
    for i in range(3):
        ref = factory(params={"sigma": float(sa.samples[i, 0])},
                      config=jx.ModelConfig(seed=1000 + i)).run()
        assert float(res["mean_x"][i]) == pytest.approx(float(ref["mean_x"][-1]), rel=1e-6)
    assert torch.all(res["missing"] == 0)


def _sir_factory(steps_hook=False):
    import jaxabm_gb300 as jx

    class HookedSIR(jx.SIRModel):
        """Same model with a no-op step hook: not batchable, runs one by one."""

        def step(self):
            pass

    cls = HookedSIR if steps_hook else jx.SIRModel

    def factory(params=None, config=None):
        p = {"n": 1500, "m": 3, "initial_infected": 0.02}
        p.update(params or {})
        return cls(p, seed=config.seed)
    return factory


def test_es_population_batched_equals_serial(cuda):
    """One ES iteration: the 20 x 2 models of the population run as one ensemble and give
    the same losses, best parameters and next population as the models run one by one."""
    import jaxabm_gb300 as jx
    kw = dict(initial_params={"beta": 0.1, "gamma": 0.2}, target_metrics={"R": 900.0},
              param_bounds={"beta": (0.01, 0.4), "gamma": (0.05, 0.5)}, max_iterations=1,
              method="es", evaluation_steps=20, num_evaluation_runs=2, seed=7)
    a = jx.ModelCalibrator(_sir_factory(), **kw)
    b = jx.ModelCalibrator(_sir_factory(steps_hook=True), **kw)
    assert torch.equal(a.es_population, b.es_population)
    pa, pb = a.calibrate(verbose=False), b.calibrate(verbose=False)
    assert a.batched_evaluations == 1 and b.batched_evaluations == 0
    assert pa == pb and a.loss_history == b.loss_history
    assert torch.equal(a.es_population, b.es_population)
    assert torch.equal(a.key, b.key)


@pytest.mark.parametrize("method", ["pso", "cem"])
def test_population_methods_run_batched(cuda, method):
    import jaxabm_gb300 as jx
    c = jx.ModelCalibrator(_sir_factory(), {"beta": 0.1, "gamma": 0.2}, {"R": 900.0},
                           param_bounds={"beta": (0.01, 0.4), "gamma": (0.05, 0.5)},
                           max_iterations=2, method=method, evaluation_steps=20,
                           num_evaluation_runs=1, seed=3)
    best = c.calibrate(verbose=False)
    assert c.batched_evaluations == 2
    assert len(c.loss_history) == 2 and c.loss_history[1] <= c.loss_history[0]
    tol = 1e-6  # bounds are float32 values
    assert 0.01 - tol <= best["beta"] <= 0.4 + tol and 0.05 - tol <= best["gamma"] <= 0.5 + tol
    hist = c.get_calibration_history()
    assert len(hist["params"]) == 2


def test_calibrator_random_walk_population_is_batched(cuda):
    import jaxabm_gb300 as jx

    def factory(params=None, config=None):
        p = {"n": 200}
        p.update(params or {})
        return jx.RandomWalkModel(p, seed=config.seed)

    c = jx.ModelCalibrator(factory, {"sigma": 0.02}, {"mean_x": 0.5},
                           param_bounds={"sigma": (0.001, 0.1)}, max_iterations=1,
                           method="es", evaluation_steps=3, num_evaluation_runs=1, seed=1)
    c.calibrate(verbose=False)
    assert c.batched_evaluations == 1 and len(c.loss_history) == 1
