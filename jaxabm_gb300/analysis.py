"""Sensitivity analysis over model parameters, run on the ensemble engine.

``SensitivityAnalysis`` keeps the reference's interface and sampling
(jaxabm/analysis.py:23-203): Latin-hypercube samples drawn with ``jax.random`` semantics,
one model per sample built by ``model_factory(params=..., config=ModelConfig(seed=1000 + i))``,
the last value of each metric of interest, and squared correlation coefficients as the
sensitivity indices.  The reference runs the samples one after another; here, when every
sample's model is a batchable SIR model, all of them run as one ensemble (one CUDA-graph
replay for every member and step, ``sir.run_ensemble``) and each member's result equals
that model's own ``run()``.  Other models run one by one, as in the reference.
"""

from typing import Any, Callable, Dict, List, Tuple

import numpy as np
import torch

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
        (jaxabm/analysis.py:97-165).  Batchable SIR models run as one ensemble."""
        from .sir import run_ensemble
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
