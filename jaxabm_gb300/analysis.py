"""Sensitivity analysis and population-based calibration, run on the ensemble engine.

``SensitivityAnalysis`` keeps the reference's interface and sampling
(jaxabm/analysis.py:23-203): Latin-hypercube samples drawn with ``jax.random`` semantics,
one model per sample built by ``model_factory(params=..., config=ModelConfig(seed=1000 + i))``,
the last value of each metric of interest, and squared correlation coefficients as the
sensitivity indices.  The reference runs the samples one after another; here, when every
sample's model belongs to a batchable family (SIR, random walk, Schelling, opinion; see
``batching.run_ensemble``), all of them run as one ensemble and each member's result
equals that model's own ``run()``.  Other models run one by one, as in the reference.
``ModelCalibrator`` evaluates each iteration's population (every candidate times every
evaluation run) the same way.
"""

from typing import Any, Callable, Dict, List, Tuple

import numpy as np
import torch

from . import _dev
from . import random as jr
from .core import ModelConfig


def _last(value):
    """The reference's rule for a metric's result: last entry of a sequence, else itself
    (jaxabm/analysis.py:140-150)."""
    if hasattr(value, "__len__") and not isinstance(value, str):
        return value[-1]
    return value


def _as_dict(results):
    return results._data if hasattr(results, "_data") else results


class SensitivityAnalysis:
    """Parameter sensitivity of a model's metrics (jaxabm/analysis.py:23-203).

    Attributes: ``model_factory``, ``param_ranges`` (name -> (min, max)),
    ``metrics_of_interest``, ``num_samples``, ``key`` (device key, advanced by sampling),
    ``samples`` (float32 tensor ``(num_samples, num_params)``), ``results`` (metric ->
    float32 tensor ``(num_samples,)``, after ``run``) and ``batched`` (whether ``run``
    went through the ensemble engine).
    """

    def __init__(self, model_factory: Callable[..., Any],
                 param_ranges: Dict[str, Tuple[float, float]],
                 metrics_of_interest: List[str], num_samples: int = 100, seed: int = 0):
        self.model_factory = model_factory
        self.param_ranges = param_ranges
        self.metrics_of_interest = metrics_of_interest
        self.num_samples = num_samples
        self.key = jr.PRNGKey(seed)
        self.samples = self._generate_lhs_samples()
        self.results = None
        self.batched = False

    def _next_key(self):
        pair = jr.split(self.key, 2)
        self.key = pair[0].contiguous()
        return pair[1].contiguous()

    def _generate_lhs_samples(self) -> torch.Tensor:
        """Latin-hypercube samples (jaxabm/analysis.py:67-95): stratum starts ``i / n`` in
        float32, a jitter ``uniform(subkey, (n,)) / n`` added, one ``permutation`` of those
        points per parameter (a fresh subkey each), then scaled by ``max - min`` and shifted
        by ``min``."""
        n = int(self.num_samples)
        jitter = jr.uniform(self._next_key(), (n,))
        # Tensor divisors: torch turns division by a host scalar into a multiplication by
        # its reciprocal, which rounds differently from the IEEE division JAX does.
        div = torch.full_like(jitter, float(n))
        points = torch.arange(n, dtype=torch.float32, device=jitter.device) / div
        points = points + jitter / div
        cols = [jr.permutation(self._next_key(), points) for _ in self.param_ranges]
        samples = (torch.stack(cols, dim=1) if cols
                   else torch.zeros((n, 0), dtype=torch.float32, device=jitter.device))
        for i, (lo, hi) in enumerate(self.param_ranges.values()):
            samples[:, i] *= np.float32(hi - lo)
            samples[:, i] += np.float32(lo)
        return samples

    def _models(self):
        names = list(self.param_ranges.keys())
        host = self.samples.cpu().numpy()
        models = []
        for i in range(self.num_samples):
            params = {name: float(host[i, j]) for j, name in enumerate(names)}
            models.append((params, self.model_factory(params=params,
                                                      config=ModelConfig(seed=i + 1000))))
        return models

    def run(self, verbose: bool = True) -> Dict[str, torch.Tensor]:
        """Run one model per sample and collect the last value of each metric of interest
        (jaxabm/analysis.py:97-165).  Batchable models run as one ensemble."""
        from .batching import run_ensemble
        if verbose:
            print(f"Running sensitivity analysis with {self.num_samples} samples...")
        pairs = self._models()
        runs = run_ensemble([m for _, m in pairs]) if pairs else []
        self.batched = runs is not None and len(pairs) > 0
        if runs is None:
            runs = []
            for i, (params, model) in enumerate(pairs):
                if verbose:
                    print(f"\nSample {i + 1}/{self.num_samples}")
                    print("Parameters: " + ", ".join(f"{k}={v:.4f}" for k, v in params.items()))
                runs.append(model.run())
        values = {m: np.zeros(self.num_samples, dtype=np.float32)
                  for m in self.metrics_of_interest}
        for i, res in enumerate(runs):
            data = _as_dict(res)
            for metric in self.metrics_of_interest:
                if metric in data and data[metric] is not None:
                    values[metric][i] = float(_last(data[metric]))
        self.results = {m: torch.from_numpy(v) for m, v in values.items()}
        if verbose:
            print("\nSensitivity analysis complete!")
        return self.results

    def sobol_indices(self) -> Dict[str, Dict[str, float]]:
        """Squared correlation of each parameter's samples with each metric, the reference's
        proxy for first-order Sobol indices (jaxabm/analysis.py:167-203): both standardised
        with the population standard deviation plus 1e-8."""
        if self.results is None:
            raise ValueError("Must run sensitivity analysis before calculating indices")
        samples = self.samples.detach().cpu().numpy().astype(np.float32)
        indices = {}
        for metric, vals in self.results.items():
            v = np.asarray(vals.detach().cpu().numpy() if torch.is_tensor(vals) else vals,
                           dtype=np.float32)
            v_norm = (v - v.mean()) / (v.std() + np.float32(1e-8))
            per_param = {}
            for i, name in enumerate(self.param_ranges):
                s = samples[:, i]
                s_norm = (s - s.mean()) / (s.std() + np.float32(1e-8))
                per_param[name] = float(np.mean(s_norm * v_norm) ** 2)
            indices[metric] = per_param
        return indices


def _evaluate_models(models, steps):
    """Run ``models`` for ``steps`` steps each: batchable models as one ensemble
    (``batching.run_ensemble``), anything else one by one.  Returns (results, batched)."""
    from .batching import run_ensemble
    for m in models:
        if hasattr(m, "steps"):
            m.steps = steps
    runs = run_ensemble(models) if models else []
    if runs is not None:
        return runs, bool(models)
    return [m.run(steps=steps) for m in models], False


class ModelCalibrator:
    """Calibration of model parameters (jaxabm/analysis.py:290-1580): gradient methods
    ``"adam"`` and ``"sgd"`` and population methods ``"es"``, ``"pso"`` and ``"cem"``.

    The constructor, ``calibrate``, the loss functions, the robust evaluation (mean metrics
    over ``num_evaluation_runs`` runs with seeds ``randint(subkey, (), 0, 1_000_000)``,
    normalised loss, 95 % intervals) and the update rules follow the reference.  What
    changes is how a population is evaluated: the reference runs its ``population x runs``
    models one after another; here every candidate of an iteration is drawn first (the key
    chain advances in the reference's order) and, for SIR models, all of them run as one
    ensemble.  ``batched_evaluations`` counts the iterations that did.

    Gradient methods follow ``_calibrate_gradient`` (jaxabm/analysis.py:1309-1394): the
    loss of a run with ``ModelConfig(seed=42)`` and its gradient, an Adam (beta1 0.9, beta2
    0.999, eps 1e-8) or SGD update, clipping to the bounds, a robust evaluation, history,
    and early stopping on ``tolerance`` and ``patience``.  The reference differentiates
    ``model.run`` with ``jit(grad(loss_fn))`` (:489-531); here the model must be
    differentiable on the engine -- it provides ``final_metrics_vjp`` (``OpinionModel``: the
    hand-written adjoint kernel with checkpoints) -- and the loss's derivative with respect
    to the final metrics is taken on the host.  The reinforcement-learning and Bayesian
    methods are not agent-step work and are not provided.
    """

    POPULATION_METHODS = ("es", "pso", "cem")
    GRADIENT_METHODS = ("adam", "sgd")

    def __init__(self, model_factory, initial_params: Dict[str, float],
                 target_metrics: Dict[str, float], param_bounds=None, metrics_weights=None,
                 learning_rate: float = 0.01, max_iterations: int = 100, method: str = "adam",
                 loss_type: str = "mse", evaluation_steps: int = 50,
                 num_evaluation_runs: int = 3, tolerance: float = 1e-6, patience: int = 10,
                 seed: int = 0):
        self.model_factory = model_factory
        self.params = dict(initial_params)
        self.target_metrics = target_metrics
        self.param_bounds = param_bounds or {k: (0.01, 10.0) for k in initial_params}
        self.metrics_weights = metrics_weights or {k: 1.0 for k in target_metrics}
        self.learning_rate = learning_rate
        self.max_iterations = max_iterations
        self.method = method
        self.loss_type = loss_type
        self.evaluation_steps = evaluation_steps
        self.num_evaluation_runs = num_evaluation_runs
        self.tolerance = tolerance
        self.patience = patience
        self._check_method()
        self.key = jr.PRNGKey(seed)
        self.loss_history: List[float] = []
        self.param_history: List[Dict[str, float]] = []
        self.confidence_intervals: List[Dict[str, Tuple[float, float]]] = []
        self.best_params = dict(initial_params)
        self.best_loss = float("inf")
        self.batched_evaluations = 0
        self._setup_optimization_method()

    # -- key chain ------------------------------------------------------------------------

    def _split(self, num=2):
        keys = jr.split(self.key, num)
        self.key = keys[0].contiguous()
        return [keys[i].contiguous() for i in range(1, num)]

    def _names(self):
        return list(self.params.keys())

    def _clip(self, pop):
        """Clip column i to the i-th entry of ``param_bounds`` (the reference pairs the
        columns with the bounds in insertion order)."""
        for i, (lo, hi) in enumerate(self.param_bounds.values()):
            pop[..., i] = torch.clamp(pop[..., i], float(lo), float(hi))
        return pop

    # -- setup (jaxabm/analysis.py:376-399, 533-597) --------------------------------------

    def _check_method(self):
        if self.method not in self.POPULATION_METHODS + self.GRADIENT_METHODS:
            known = ("bayesian", "q_learning", "policy_gradient", "actor_critic",
                     "multi_agent_rl", "dqn")
            if self.method in known:
                raise NotImplementedError(
                    f"calibration method {self.method!r} is not provided by this engine; "
                    f"methods: {', '.join(self.GRADIENT_METHODS + self.POPULATION_METHODS)}")
            raise ValueError(f"Unknown calibration method: {self.method}")

    def _setup_optimization_method(self):
        self._check_method()
        n = len(self.params)
        init = torch.tensor([float(self.params[k]) for k in self._names()],
                            dtype=torch.float32)
        if self.method in self.GRADIENT_METHODS:
            # jaxabm/analysis.py:524-531
            self.adam_m = np.zeros(n)
            self.adam_v = np.zeros(n)
            self.adam_beta1, self.adam_beta2, self.adam_eps = 0.9, 0.999, 1e-8
            self.adam_t = 0
        elif self.method == "es":
            self.es_population_size, self.es_sigma, self.es_elite_ratio = 20, 0.1, 0.2
            (sub,) = self._split()
            pop = jr.normal(sub, (self.es_population_size, n)) * self.es_sigma
            self.es_population = self._clip(pop + init.to(pop.device)[None, :])
        elif self.method == "pso":
            self.pso_population_size, self.pso_w, self.pso_c1, self.pso_c2 = 20, 0.7, 1.5, 1.5
            (sub,) = self._split()
            pos = jr.uniform(sub, (self.pso_population_size, n))
            for i, (lo, hi) in enumerate(self.param_bounds.values()):
                pos[:, i] *= np.float32(hi - lo)
                pos[:, i] += np.float32(lo)
            self.pso_positions = pos
            (sub,) = self._split()
            self.pso_velocities = jr.normal(sub, (self.pso_population_size, n)) * 0.1
            self.pso_personal_best = pos.clone()
            self.pso_personal_best_scores = torch.full((self.pso_population_size,),
                                                       float("inf"), device=pos.device)
            self.pso_global_best = pos[0].clone()
            self.pso_global_best_score = float("inf")
        else:
            self.cem_population_size, self.cem_elite_ratio, self.cem_noise_decay = 50, 0.2, 0.99
            self.cem_mean = init.to(_dev.device())
            self.cem_std = torch.ones(n, dtype=torch.float32, device=self.cem_mean.device) * 0.5

    # -- losses (jaxabm/analysis.py:401-487) ----------------------------------------------

    def _compute_loss(self, metrics: Dict[str, float]) -> float:
        loss = 0.0
        for metric, target in self.target_metrics.items():
            if metric not in metrics:
                continue
            value, weight = metrics[metric], self.metrics_weights[metric]
            if self.loss_type == "mse":
                metric_loss = (value - target) ** 2
            elif self.loss_type == "mae":
                metric_loss = abs(value - target)
            elif self.loss_type == "huber":
                residual = abs(value - target)
                metric_loss = 0.5 * residual ** 2 if residual <= 1.0 else residual - 0.5
            elif self.loss_type == "relative":
                metric_loss = abs(value - target) / (abs(target) + 1e-8)
            else:
                raise ValueError(f"Unknown loss type: {self.loss_type}")
            loss += weight * metric_loss
        return loss

    def _loss_gradient(self, metrics: Dict[str, float]) -> Dict[str, float]:
        """d loss / d metric value of :meth:`_compute_loss` for each target metric present
        (derivatives of the four loss types; |x| and the Huber kink use sign(x))."""
        out = {}
        for metric, target in self.target_metrics.items():
            if metric not in metrics:
                continue
            r, w = metrics[metric] - target, self.metrics_weights[metric]
            if self.loss_type == "mse":
                d = 2.0 * r
            elif self.loss_type == "mae":
                d = float(np.sign(r))
            elif self.loss_type == "huber":
                d = r if abs(r) <= 1.0 else float(np.sign(r))
            elif self.loss_type == "relative":
                d = float(np.sign(r)) / (abs(target) + 1e-8)
            else:
                raise ValueError(f"Unknown loss type: {self.loss_type}")
            out[metric] = w * d
        return out

    def loss_and_grad(self, params_flat):
        """(loss, gradient float64[n_params]) of the reference's gradient objective at
        ``params_flat``: the model built with ``ModelConfig(seed=42)``, run for
        ``evaluation_steps`` steps, loss of the last value of each target metric (0 for a
        metric the model does not report), differentiated through the model's adjoint."""
        names = self._names()
        params = {name: float(params_flat[i]) for i, name in enumerate(names)}
        model = self.model_factory(params=params, config=ModelConfig(seed=42))
        if not hasattr(model, "final_metrics_vjp"):
            raise NotImplementedError(
                f"gradient calibration needs a differentiable model (one with "
                f"final_metrics_vjp, such as OpinionModel); {type(model).__name__} has none")
        final, vjp = model.final_metrics_vjp(names, steps=self.evaluation_steps)
        metrics = {m: float(final.get(m, 0.0)) for m in self.target_metrics}
        loss = self._compute_loss(metrics)
        grads = vjp(self._loss_gradient(metrics))
        return float(loss), np.array([grads[name] for name in names], dtype=np.float64)

    def _compute_normalized_loss(self, metrics: Dict[str, float]) -> float:
        total = 0.0
        for metric, target in self.target_metrics.items():
            if metric in metrics:
                total += (abs(metrics[metric] - target) / (abs(target) + 1e-8)) ** 2
        return float(total)

    # -- evaluation (jaxabm/analysis.py:434-476) ------------------------------------------

    def _metric_values(self, results):
        data = _as_dict(results)
        out = {}
        for metric in self.target_metrics:
            v = data[metric] if metric in data else None
            if v is not None and hasattr(v, "__len__") and len(v) > 0:
                out[metric] = float(v[-1])
            else:
                out[metric] = 0.0
        return out

    def _summarise(self, runs):
        """Normalised loss and 95 % intervals of one candidate's runs."""
        means, cis = {}, {}
        for metric in self.target_metrics:
            vals = np.array([r[metric] for r in runs], dtype=np.float32)
            mean, std = float(vals.mean()), float(vals.std())
            half = 1.96 * std / float(np.sqrt(np.float32(len(vals))))
            means[metric] = mean
            cis[metric] = (mean - half, mean + half)
        return self._compute_normalized_loss(means), cis

    def _evaluate_population(self, candidates: List[Dict[str, float]]):
        """(loss, intervals) per candidate.  Seeds are drawn candidate by candidate, run by
        run, as the reference's serial loop draws them; then every model runs."""
        models = []
        for params in candidates:
            for _ in range(self.num_evaluation_runs):
                (sub,) = self._split()
                seed = int(jr.randint(sub, (), 0, 1_000_000).item())
                models.append(self.model_factory(params=params, config=ModelConfig(seed=seed)))
        results, batched = _evaluate_models(models, self.evaluation_steps)
        self.batched_evaluations += int(batched)
        R = self.num_evaluation_runs
        out = []
        for c in range(len(candidates)):
            runs = [self._metric_values(r) for r in results[c * R:(c + 1) * R]]
            out.append(self._summarise(runs))
        return out

    def _evaluate_params_robust(self, params: Dict[str, float]):
        return self._evaluate_population([params])[0]

    def _rows(self, pop):
        host = pop.detach().cpu().numpy()
        return [{name: float(host[i, j]) for j, name in enumerate(self._names())}
                for i in range(host.shape[0])]

    # -- calibration loops (jaxabm/analysis.py:1281-1580) --------------------------------

    def calibrate(self, verbose: bool = True) -> Dict[str, float]:
        if verbose:
            print(f"Starting calibration with {self.method} method...")
            print(f"Target metrics: {self.target_metrics}")
            print(f"Parameter bounds: {self.param_bounds}")
        return {"adam": self._calibrate_gradient, "sgd": self._calibrate_gradient,
                "es": self._calibrate_evolution_strategies,
                "pso": self._calibrate_particle_swarm,
                "cem": self._calibrate_cross_entropy}[self.method](verbose)

    def _calibrate_gradient(self, verbose: bool) -> Dict[str, float]:
        """Adam or SGD on the adjoint gradient (jaxabm/analysis.py:1309-1394)."""
        names = self._names()
        params_flat = np.array([float(self.params[k]) for k in names], dtype=np.float64)
        no_improvement = 0
        for it in range(self.max_iterations):
            if verbose:
                print(f"\nIteration {it + 1}/{self.max_iterations}")
            _, grads = self.loss_and_grad(params_flat)
            if np.any(np.isnan(grads)):
                if verbose:
                    print("NaN gradients detected, stopping optimization")
                break
            if self.method == "adam":
                self.adam_t += 1
                self.adam_m = self.adam_beta1 * self.adam_m + (1 - self.adam_beta1) * grads
                self.adam_v = self.adam_beta2 * self.adam_v + (1 - self.adam_beta2) * grads ** 2
                m_hat = self.adam_m / (1 - self.adam_beta1 ** self.adam_t)
                v_hat = self.adam_v / (1 - self.adam_beta2 ** self.adam_t)
                params_flat = params_flat - self.learning_rate * m_hat / (np.sqrt(v_hat)
                                                                          + self.adam_eps)
            else:
                params_flat = params_flat - self.learning_rate * grads
            for i, (lo, hi) in enumerate(self.param_bounds.values()):
                params_flat[i] = min(max(params_flat[i], float(lo)), float(hi))
            for i, name in enumerate(names):
                self.params[name] = float(params_flat[i])
            loss, ci = self._evaluate_params_robust(self.params)
            self.param_history.append(dict(self.params))
            self.loss_history.append(loss)
            self.confidence_intervals.append(ci)
            if loss < self.best_loss:
                self.best_loss = loss
                self.best_params = dict(self.params)
                no_improvement = 0
            else:
                no_improvement += 1
            if verbose:
                print(f"Loss: {loss:.6f} (best: {self.best_loss:.6f})")
            if loss < self.tolerance:
                if verbose:
                    print("Converged: loss below tolerance")
                break
            if no_improvement >= self.patience:
                if verbose:
                    print("Early stopping: no improvement")
                break
        return self.best_params

    def _elite_step(self, pop, verbose, iteration):
        scores = [loss for loss, _ in self._evaluate_population(self._rows(pop))]
        fitness = torch.tensor(scores, dtype=torch.float32)
        n_elite = int(pop.shape[0] * (self.es_elite_ratio if self.method == "es"
                                      else self.cem_elite_ratio))
        elite_idx = torch.sort(fitness, stable=True).indices[:n_elite]
        elite = pop[elite_idx.to(pop.device)]
        best_idx = int(elite_idx[0])
        best_loss = float(fitness[best_idx])
        if best_loss < self.best_loss:
            self.best_loss = best_loss
            self.best_params = self._rows(pop[best_idx:best_idx + 1])[0]
        if verbose:
            print(f"\nIteration {iteration + 1}/{self.max_iterations}")
            print(f"Best loss: {best_loss:.6f}")
        return elite, best_loss

    def _calibrate_evolution_strategies(self, verbose: bool) -> Dict[str, float]:
        for it in range(self.max_iterations):
            elite, best_loss = self._elite_step(self.es_population, verbose, it)
            (sub,) = self._split()
            mean = elite.mean(dim=0)
            noise = jr.normal(sub, tuple(self.es_population.shape)) * np.float32(self.es_sigma)
            self.es_population = self._clip(mean[None, :] + noise)
            self.loss_history.append(best_loss)
            self.param_history.append(dict(self.best_params))
            self.es_sigma *= 0.995
            if best_loss < self.tolerance:
                if verbose:
                    print("Converged: loss below tolerance")
                break
        return self.best_params

    def _calibrate_cross_entropy(self, verbose: bool) -> Dict[str, float]:
        n = len(self.params)
        for it in range(self.max_iterations):
            (sub,) = self._split()
            pop = jr.normal(sub, (self.cem_population_size, n))
            pop = self._clip(pop * self.cem_std[None, :] + self.cem_mean[None, :])
            elite, best_loss = self._elite_step(pop, verbose, it)
            self.cem_mean = elite.mean(dim=0)
            self.cem_std = elite.std(dim=0, unbiased=False) + np.float32(1e-6)
            self.loss_history.append(best_loss)
            self.param_history.append(dict(self.best_params))
            self.cem_std = self.cem_std * np.float32(self.cem_noise_decay)
            if best_loss < self.tolerance:
                if verbose:
                    print("Converged: loss below tolerance")
                break
        return self.best_params

    def _calibrate_particle_swarm(self, verbose: bool) -> Dict[str, float]:
        for it in range(self.max_iterations):
            rows = self._rows(self.pso_positions)
            evals = self._evaluate_population(rows)
            for i, (loss, _) in enumerate(evals):
                if loss < float(self.pso_personal_best_scores[i]):
                    self.pso_personal_best_scores[i] = loss
                    self.pso_personal_best[i] = self.pso_positions[i]
                if loss < self.pso_global_best_score:
                    self.pso_global_best_score = loss
                    self.pso_global_best = self.pso_positions[i].clone()
                    self.best_loss = loss
                    self.best_params = dict(rows[i])
            sub1, sub2 = self._split(3)
            shape = tuple(self.pso_velocities.shape)
            r1, r2 = jr.uniform(sub1, shape), jr.uniform(sub2, shape)
            cognitive = np.float32(self.pso_c1) * r1 * (self.pso_personal_best - self.pso_positions)
            social = np.float32(self.pso_c2) * r2 * (self.pso_global_best[None, :] -
                                                     self.pso_positions)
            self.pso_velocities = np.float32(self.pso_w) * self.pso_velocities + cognitive + social
            self.pso_positions = self._clip(self.pso_positions + self.pso_velocities)
            self.loss_history.append(float(self.pso_global_best_score))
            self.param_history.append(dict(self.best_params))
            if verbose:
                print(f"\nIteration {it + 1}/{self.max_iterations}")
                print(f"Best loss: {self.pso_global_best_score:.6f}")
            if self.pso_global_best_score < self.tolerance:
                if verbose:
                    print("Converged: loss below tolerance")
                break
        return self.best_params

    def get_calibration_history(self) -> Dict[str, List[Any]]:
        return {"loss": self.loss_history, "params": self.param_history,
                "confidence_intervals": self.confidence_intervals}
