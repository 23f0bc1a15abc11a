"""Utilities (mirrors the parts of jaxabm/utils.py the API surface needs)."""

from typing import Any

import numpy as np
import torch


def convert_to_numpy(data: Any) -> Any:
    """Device tensors -> NumPy arrays, recursively (jaxabm/utils.py:17-38)."""
    if isinstance(data, dict):
        return {k: convert_to_numpy(v) for k, v in data.items()}
    if isinstance(data, list):
        return [convert_to_numpy(v) for v in data]
    if isinstance(data, tuple):
        return tuple(convert_to_numpy(v) for v in data)
    if isinstance(data, torch.Tensor):
        return data.detach().cpu().numpy()
    return data


def format_time(seconds: float) -> str:
    """Human-readable duration (jaxabm/utils.py:54-73)."""
    if seconds < 60:
        return f"{seconds:.2f}s"
    if seconds < 3600:
        minutes = int(seconds / 60)
        return f"{minutes}m {seconds % 60:.2f}s"
    hours = int(seconds / 3600)
    minutes = int((seconds % 3600) / 60)
    return f"{hours}h {minutes}m {seconds % 60:.2f}s"


def mean_over_runs(results_list):
    """Element-wise mean of metric lists over runs (jaxabm/utils.py:76-103)."""
    if not results_list:
        return {}
    keys = results_list[0].keys()
    return {k: list(np.mean(np.array([r[k] for r in results_list], dtype=float), axis=0))
            for k in keys}
