"""Model configuration (mirrors jaxabm/core.py:55-87) and framework info."""


class ModelConfig:
    """Configuration for model execution (jaxabm/core.py:55-87).

    Attributes:
        seed: random seed (``PRNGKey(seed)`` starts the key chain)
        steps: number of simulation steps to run
        track_history: whether ``run`` records per-step metrics
        collect_interval: record every ``collect_interval``-th step
    """

    def __init__(self, seed: int = 0, steps: int = 100, track_history: bool = True,
                 collect_interval: int = 1):
        self.seed = seed
        self.steps = steps
        self.track_history = track_history
        self.collect_interval = collect_interval


_VERBOSE = [True]


def set_verbose(flag: bool) -> None:
    """Turn the reference's run-time prints (``Ran N steps in ...``) on or off."""
    _VERBOSE[0] = bool(flag)


def verbose() -> bool:
    return _VERBOSE[0]


def has_cuda() -> bool:
    import torch
    return torch.cuda.is_available()


def show_info() -> None:
    """Print version, device and registered step kernels (jaxabm/core.py:89-117)."""
    from . import __version__
    from .registry import registered
    print(f"jaxabm_gb300 v{__version__}")
    print("GB300-native agent-step engine (CUDA sm_103a)")
    if has_cuda():
        import torch
        print(f"Device: {torch.cuda.get_device_name()}")
    else:
        print("No CUDA device visible: models cannot run here.")
    print("Registered step kernels:")
    for cls, k in registered().items():
        print(f"  - {cls.__name__}: {k.name}")
