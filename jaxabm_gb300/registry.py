"""Step-kernel registry: binds an Agent (or AgentType) class to its fused CUDA step.

The reference runs any traced Python ``Agent.step`` through ``jax.vmap``
(jaxabm/agent.py:168-177, jaxabm/agentpy.py:199-227).  This engine has no tracing compiler:
each agent class runs on a hand-written kernel registered for it.  A class with no
registered kernel is rejected with :class:`UnregisteredAgentError` when its collection is
initialised, before any launch; there is no CPU or eager fallback.
"""

from typing import Dict, Type


class UnregisteredAgentError(TypeError):
    """The agent class has no registered step kernel."""


class StepKernel:
    """Interface of a registered fused step.

    Attributes:
        name: kernel family name (``"randomwalk"``, ``"sir"``, ...)
        attributes: SoA attribute names the kernel owns
        metrics: names of the per-step metrics the kernel reduces in its epilogue
        params: parameter defaults (overridden by ``add_agents`` kwargs or AgentType
            attributes of the same name)
        independent: the step reads only this collection's own states and the static
            environment it was given, so consecutive steps can run as one fused launch
    """

    name = ""
    attributes: tuple = ()
    metrics: tuple = ()
    params: dict = {}
    independent = True

    def resolve_params(self, given: dict) -> dict:
        out = dict(self.params)
        for k in self.params:
            if given is not None and k in given:
                out[k] = given[k]
        return out

    def init(self, n, init_key, params, env):
        """Return the initial SoA states (dict of CUDA tensors) for ``n`` agents."""
        raise NotImplementedError

    def step(self, states, coll_key, params, env):
        """One synchronous step.  Returns (new_states, metrics row tensor or None)."""
        raise NotImplementedError

    def run(self, states, coll_keys, params, env):
        """``coll_keys.shape[0]`` steps.  Returns (new_states, metrics [T, m] or None)."""
        metrics = []
        for t in range(coll_keys.shape[0]):
            states, m = self.step(states, coll_keys[t], params, env)
            if m is not None:
                metrics.append(m)
        import torch
        return states, (torch.stack(metrics) if metrics else None)


_REGISTRY: Dict[type, StepKernel] = {}
_HOOKS = ("setup", "step", "init_state", "update")


def register_step(agent_cls: Type = None, kernel: StepKernel = None):
    """Register ``kernel`` as the fused step of ``agent_cls``.

    Usable directly (``register_step(MyAgent, MyKernel())``) or as a class decorator
    (``@register_step(kernel=MyKernel())``).
    """
    if agent_cls is None:
        def deco(cls):
            register_step(cls, kernel)
            return cls
        return deco
    if not isinstance(agent_cls, type):
        raise TypeError("register_step expects an agent class")
    if not isinstance(kernel, StepKernel):
        raise TypeError("kernel must be a StepKernel instance")
    _REGISTRY[agent_cls] = kernel
    return agent_cls


def unregister_step(agent_cls: Type) -> None:
    _REGISTRY.pop(agent_cls, None)


def registered() -> Dict[type, StepKernel]:
    return dict(_REGISTRY)


def agent_class_of(agent_type) -> type:
    """The user-facing class behind an AgentWrapper, AgentType instance or class."""
    cls = getattr(agent_type, "agent_class", None)
    if isinstance(cls, type):
        return cls
    return agent_type if isinstance(agent_type, type) else type(agent_type)


def lookup(agent_type) -> StepKernel:
    """Kernel registered for ``agent_type``'s class.

    A subclass of a registered class is accepted only if it overrides none of
    ``setup``/``step``/``init_state``/``update`` (its behaviour is then the base's).
    """
    cls = agent_class_of(agent_type)
    k = _REGISTRY.get(cls)
    if k is not None:
        return k
    for base in cls.__mro__[1:]:
        kb = _REGISTRY.get(base)
        if kb is None:
            continue
        if all(getattr(cls, h, None) is getattr(base, h, None) for h in _HOOKS):
            return kb
        break
    raise UnregisteredAgentError(
        f"agent class {cls.__name__} has no registered step kernel; register one with "
        "jaxabm_gb300.register_step (there is no CPU fallback)")
