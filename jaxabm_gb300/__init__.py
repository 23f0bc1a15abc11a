"""jaxabm_gb300: a GB300-native agent-step engine behind the JaxABM API.

Drop-in surface of ``jaxabm`` (jaxabm/__init__.py:57-156) for the agent-step path:
``Agent, AgentList, Environment, Grid, Network, Model, Results`` (AgentPy-like API) and
``AgentType, AgentCollection, JaxModel, ModelConfig`` (core API).  Agent state lives in
structure-of-arrays CUDA tensors; every step runs in hand-written sm_103a kernels behind
the C ABI of ``libjaxabm_gb300.so`` (include/jaxabm_gb300.h).  Agent classes run on the
kernel registered for them (:func:`register_step`); there is no CPU fallback.
"""

__version__ = "0.1.0"

from . import random
from ._build import build as _build_library
from ._lib import AbmError
from .agent import AgentCollection, AgentType
from .agentpy import Agent, AgentList, Environment, Grid, Model, Network, Results
from .core import ModelConfig, has_cuda, set_verbose, show_info
from .trace import set_tracing, tracing
from .model import Model as JaxModel
from .registry import StepKernel, UnregisteredAgentError, lookup, register_step, unregister_step
from .utils import convert_to_numpy, format_time

from . import randomwalk  # noqa: E402  registers RandomWalker
from .randomwalk import RandomWalker, RandomWalkModel  # noqa: E402
from . import sir  # noqa: E402  registers SIRAgent
from .sir import SIRAgent, SIRModel  # noqa: E402
from . import schelling  # noqa: E402  registers SchellingAgent
from .schelling import SchellingAgent, SchellingModel  # noqa: E402
from . import opinion  # noqa: E402  registers OpinionAgent
from .opinion import OpinionAgent, OpinionModel  # noqa: E402
from .analysis import ModelCalibrator, SensitivityAnalysis  # noqa: E402


def build(force: bool = False, checked: bool = False) -> str:
    """Compile ``libjaxabm_gb300.so`` for sm_103a (in-tree) and return its path; with
    ``checked``, the range-checked ``libjaxabm_gb300_checked.so`` (``JAXABM_CHECKED=1``
    makes the package load it)."""
    return _build_library(force=force, checked=checked)


def has_jax() -> bool:
    """The reference's availability check; this engine does not use JAX."""
    return False


def jax_available() -> bool:
    return False


def cuda_available() -> bool:
    return has_cuda()


__all__ = [
    "Agent", "AgentList", "Environment", "Grid", "Network", "Model", "Results",
    "AgentType", "AgentCollection", "JaxModel", "ModelConfig",
    "StepKernel", "UnregisteredAgentError", "register_step", "unregister_step", "lookup",
    "convert_to_numpy", "format_time", "random", "build", "show_info", "set_verbose", "set_tracing", "tracing",
    "RandomWalker", "RandomWalkModel", "AbmError", "SensitivityAnalysis", "ModelCalibrator",
]
