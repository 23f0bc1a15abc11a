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


def _bare_calibrator(**kw):
    from jaxabm_gb300.analysis import ModelCalibrator
    c = ModelCalibrator.__new__(ModelCalibrator)
    c.target_metrics = kw.get("targets", {"a": 2.0, "b": -1.0})
    c.metrics_weights = kw.get("weights", {"a": 1.0, "b": 0.5})
    c.loss_type = kw.get("loss_type", "mse")
    return c


@pytest.mark.parametrize("loss_type,want", [
    ("mse", (3.0 - 2.0) ** 2 + 0.5 * (-0.5 + 1.0) ** 2),
    ("mae", 1.0 + 0.5 * 0.5),
    ("huber", (1.0 - 0.5) + 0.5 * (0.5 * 0.5 ** 2)),
    ("relative", 1.0 / 2.0 + 0.5 * 0.5 / 1.0),
])
def test_calibrator_losses(loss_type, want):
    """The reference's loss types (jaxabm/analysis.py:401-431); Huber with delta 1."""
    c = _bare_calibrator(loss_type=loss_type)
    assert c._compute_loss({"a": 3.0, "b": -0.5, "other": 9.0}) == pytest.approx(want)


def test_calibrator_normalized_loss_and_intervals():
    c = _bare_calibrator()
    assert c._compute_normalized_loss({"a": 3.0}) == pytest.approx(0.25)
    loss, ci = c._summarise([{"a": 1.0, "b": -1.0}, {"a": 3.0, "b": -1.0}])
    assert loss == pytest.approx(0.0)
    half = 1.96 * 1.0 / np.sqrt(2)
    assert ci["a"] == pytest.approx((2.0 - half, 2.0 + half))
    assert ci["b"] == pytest.approx((-1.0, -1.0))


def test_calibrator_methods_rejected_before_any_launch():
    from jaxabm_gb300.analysis import ModelCalibrator
    with pytest.raises(ValueError):
        ModelCalibrator(None, {"beta": 0.1}, {"R": 1.0}, method="nope")
    with pytest.raises(NotImplementedError):
        ModelCalibrator(None, {"beta": 0.1}, {"R": 1.0}, method="bayesian")


@pytest.mark.parametrize("loss_type", ["mse", "mae", "huber", "relative"])
def test_calibrator_loss_gradient_matches_finite_differences(loss_type):
    c = _bare_calibrator(loss_type=loss_type)
    m = {"a": 3.3, "b": -0.4}
    g = c._loss_gradient(m)
    for k in m:
        h = 1e-6
        up, dn = dict(m), dict(m)
        up[k] += h
        dn[k] -= h
        fd = (c._compute_loss(up) - c._compute_loss(dn)) / (2 * h)
        assert g[k] == pytest.approx(fd, rel=1e-5, abs=1e-8)


class _OracleRandom:
    """The device ``jax.random`` of the package, restated on the oracle for host-only
    tests of the analysis loops (int32 key tensors, as on the device)."""

    @staticmethod
    def _np(key):
        return key.numpy().astype(np.int32).view(np.uint32).reshape(-1)

    @staticmethod
    def _t(a, dtype=torch.int32):
        a = np.asarray(a)
        if a.dtype == np.uint32:
            a = a.view(np.int32)
        return torch.from_numpy(np.ascontiguousarray(a)).to(dtype)

    def PRNGKey(self, seed):
        return self._t(tf.PRNGKey(seed))

    def split(self, key, num=2):
        return self._t(tf.split(self._np(key), num))

    def uniform(self, key, shape=()):
        return self._t(tf.uniform(self._np(key), shape).astype(np.float32), torch.float32)

    def normal(self, key, shape=()):
        return self._t(tf.normal(self._np(key), shape).astype(np.float32), torch.float32)

    def randint(self, key, shape, lo, hi):
        return self._t(tf.randint(self._np(key), shape, lo, hi))

    def permutation(self, key, x):
        out = tf.permutation(self._np(key), x.numpy() if torch.is_tensor(x) else x)
        return torch.from_numpy(np.ascontiguousarray(out))


class _ToyModel:
    """Stands in for a model: its final 'R' is a smooth function of (beta, gamma) plus a
    seed-dependent wobble, so the population methods have a minimum to find."""

    def __init__(self, params, seed):
        self.p, self.seed = params, seed

    def run(self, steps=None):
        b, g = self.p["beta"], self.p["gamma"]
        wobble = ((self.seed * 2654435761) % 1000) / 1e5
        return {"R": [0.0, 500.0 * b / g + wobble]}


@pytest.mark.parametrize("method", ["es", "pso", "cem"])
def test_calibrator_population_loops_on_host(monkeypatch, method):
    """ES, PSO and CEM loops with the oracle's random numbers and a toy model: histories
    have one entry per iteration (each iteration's best for ES and CEM, the running best
    for PSO, as in the reference), the kept best is the lowest loss seen, parameters stay
    in bounds, and the same seed repeats the same run."""
    from jaxabm_gb300 import analysis
    monkeypatch.setattr(analysis, "jr", _OracleRandom())
    monkeypatch.setattr(analysis._dev, "device", lambda: torch.device("cpu"))

    def factory(params=None, config=None):
        return _ToyModel(params, config.seed)

    def calibrate(seed):
        c = analysis.ModelCalibrator(factory, {"beta": 0.1, "gamma": 0.2}, {"R": 400.0},
                                     param_bounds={"beta": (0.01, 0.4), "gamma": (0.05, 0.5)},
                                     max_iterations=4, method=method, evaluation_steps=5,
                                     num_evaluation_runs=2, tolerance=-1.0, seed=seed)
        best = c.calibrate(verbose=False)
        return c, best

    c, best = calibrate(5)
    assert len(c.loss_history) == 4 and len(c.param_history) == 4
    if method == "pso":
        assert all(b <= a for a, b in zip(c.loss_history, c.loss_history[1:]))
    assert c.best_loss <= min(c.loss_history)
    assert 0.01 - 1e-6 <= best["beta"] <= 0.4 + 1e-6 and 0.05 - 1e-6 <= best["gamma"] <= 0.5 + 1e-6
    assert c.batched_evaluations == 0  # toy models run one by one
    c2, best2 = calibrate(5)
    assert best2 == best and c2.loss_history == c.loss_history


def test_sensitivity_analysis_on_host(monkeypatch):
    """SensitivityAnalysis end to end with the oracle's random numbers and toy models (run
    one by one): samples equal the oracle's Latin hypercube, each sample's model is built
    with seed 1000 + i, and the result is the last value of each metric."""
    from jaxabm_gb300 import analysis
    monkeypatch.setattr(analysis, "jr", _OracleRandom())
    seeds = []

    def factory(params=None, config=None):
        seeds.append(config.seed)
        return _ToyModel(params, config.seed)

    ranges = {"beta": (0.05, 0.3), "gamma": (0.1, 0.4)}
    sa = analysis.SensitivityAnalysis(factory, ranges, ["R", "missing"], num_samples=12, seed=9)
    assert np.array_equal(sa.samples.numpy(), lhs_oracle(9, 12, list(ranges.values())))
    res = sa.run(verbose=False)
    assert seeds == [1000 + i for i in range(12)] and not sa.batched
    for i in range(12):
        want = _ToyModel({"beta": float(sa.samples[i, 0]), "gamma": float(sa.samples[i, 1])},
                         1000 + i).run()["R"][-1]
        assert float(res["R"][i]) == pytest.approx(want, rel=1e-6)
    assert torch.all(res["missing"] == 0)
    idx = sa.sobol_indices()
    assert set(idx["R"]) == {"beta", "gamma"}
    assert all(0.0 <= v <= 1.0 + 1e-6 for v in idx["R"].values())
    assert idx["R"]["beta"] > 0.1 and idx["R"]["gamma"] > 0.1  # R = 500 beta / gamma


class _ToyDifferentiable:
    """A model with an analytic adjoint: final metric m1 = mu^2 + 3 eps, m2 = mu eps (the
    seed adds a small offset to both), so the gradient loop has a known derivative."""

    def __init__(self, params, seed):
        self.p, self.seed = params, seed

    def _metrics(self):
        mu, eps = self.p["mu"], self.p["eps"]
        off = (self.seed % 7) * 1e-4
        return {"m1": mu * mu + 3 * eps + off, "m2": mu * eps + off}

    def run(self, steps=None):
        m = self._metrics()
        return {"m1": [0.0, m["m1"]], "m2": [0.0, m["m2"]]}

    def final_metrics_vjp(self, names, steps=None):
        mu, eps = self.p["mu"], self.p["eps"]

        def vjp(d):
            g = {"mu": d.get("m1", 0.0) * 2 * mu + d.get("m2", 0.0) * eps,
                 "eps": d.get("m1", 0.0) * 3 + d.get("m2", 0.0) * mu}
            return {k: g[k] for k in names}
        return self._metrics(), vjp


@pytest.mark.parametrize("method", ["adam", "sgd"])
def test_calibrator_gradient_loop_on_host(monkeypatch, method):
    """The adam / sgd loop of the reference (jaxabm/analysis.py:1309-1394) with a toy
    differentiable model: the gradient equals the chain rule through the model's adjoint,
    the first update follows the reference's formula, parameters stay in bounds, the loss
    falls, and the robust evaluation's history has one entry per iteration."""
    from jaxabm_gb300 import analysis
    monkeypatch.setattr(analysis, "jr", _OracleRandom())
    monkeypatch.setattr(analysis._dev, "device", lambda: torch.device("cpu"))

    def factory(params=None, config=None):
        return _ToyDifferentiable(params, config.seed)

    targets = {"m1": 1.0, "m2": 0.1}  # reached near mu = 0.34, eps = 0.295
    c = analysis.ModelCalibrator(factory, {"mu": 0.8, "eps": 0.5}, targets,
                                 param_bounds={"mu": (0.0, 2.0), "eps": (0.0, 1.0)},
                                 learning_rate=0.05, max_iterations=40, method=method,
                                 num_evaluation_runs=2, tolerance=-1.0, patience=100, seed=3)
    loss0, g0 = c.loss_and_grad(np.array([0.8, 0.5]))
    m = _ToyDifferentiable({"mu": 0.8, "eps": 0.5}, 42)._metrics()
    r1, r2 = m["m1"] - 1.0, m["m2"] - 0.1
    assert loss0 == pytest.approx(r1 ** 2 + r2 ** 2)
    assert g0 == pytest.approx([2 * r1 * 1.6 + 2 * r2 * 0.5, 2 * r1 * 3 + 2 * r2 * 0.8])
    best = c.calibrate(verbose=False)
    first = c.param_history[0]
    if method == "sgd":
        want = np.array([0.8, 0.5]) - 0.05 * g0
    else:  # one Adam step moves every parameter by the learning rate against its gradient
        want = np.array([0.8, 0.5]) - 0.05 * g0 / (np.abs(g0) + 1e-8)
    assert [first["mu"], first["eps"]] == pytest.approx(want.tolist(), rel=1e-9)
    assert len(c.loss_history) == 40 == len(c.confidence_intervals)
    assert c.loss_history[-1] < (0.1 if method == "adam" else 0.8) * c.loss_history[0]
    assert 0.0 <= best["mu"] <= 2.0 and 0.0 <= best["eps"] <= 1.0
    assert c.best_loss == min(c.loss_history)


def test_calibrator_gradient_needs_differentiable_model(monkeypatch):
    from jaxabm_gb300 import analysis
    monkeypatch.setattr(analysis, "jr", _OracleRandom())
    c = analysis.ModelCalibrator(lambda params=None, config=None: _ToyModel(params, 0),
                                 {"beta": 0.1, "gamma": 0.2}, {"R": 1.0}, method="sgd")
    with pytest.raises(NotImplementedError, match="differentiable"):
        c.calibrate(verbose=False)
