"""Checkpoint / resume: ``Model.state_dict()`` then ``load_state_dict()`` on a fresh model
continues bit for bit -- same per-step metrics and same agent and environment tensors as
the model that kept running, and as one uninterrupted run of all the steps.  Covers the
four registered families (random walk, Schelling with its grid in the environment, SIR
on a network, the opinion model)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _factories():
    import jaxabm_gb300 as jx
    return {
        "randomwalk": lambda: jx.RandomWalkModel({"n": 3000, "seed": 5}),
        "schelling": lambda: jx.SchellingModel({"width": 48, "height": 40, "density": 0.9},
                                               seed=2),
        "sir": lambda: jx.SIRModel({"n": 5000, "m": 4, "beta": 0.08, "gamma": 0.1,
                                    "initial_infected": 0.01}, seed=4),
        "opinion": lambda: jx.OpinionModel({"n": 2048, "degree": 16}, seed=1),
    }


def _tensors(model):
    out = {}
    for name, c in model.agent_collections.items():
        for k, v in c.states.items():
            out[f"{name}.{k}"] = v.detach().cpu().clone()
    for k, v in model._env_state.items():
        if isinstance(v, torch.Tensor):
            out[f"env.{k}"] = v.detach().cpu().clone()
    return out


def _same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert torch.equal(a[k], b[k]), k


@pytest.mark.parametrize("family", ["randomwalk", "schelling", "sir", "opinion"])
def test_resume_is_bit_identical(cuda, family):
    make = _factories()[family]
    k1, k2 = 13, 11
    a = make().core_model()
    a.run(k1)
    saved = a.state_dict()
    ra = a.run(k2)
    after_a = _tensors(a)

    b = make().core_model()
    b.load_state_dict(saved)
    rb = b.run(k2)
    assert ra.keys() == rb.keys()
    for key in ra:
        assert np.array_equal(np.asarray(ra[key]), np.asarray(rb[key])), key
    assert ra["step"] == list(range(k1 + 1, k1 + k2 + 1))
    _same(after_a, _tensors(b))

    c = make().core_model()
    rc = c.run(k1 + k2)
    _same(after_a, _tensors(c))
    for key in ra:
        assert np.array_equal(np.asarray(ra[key]), np.asarray(rc[key])[k1:]), key


def test_state_dict_is_a_copy(cuda):
    import jaxabm_gb300 as jx
    m = jx.RandomWalkModel({"n": 500, "seed": 0}).core_model()
    m.run(3)
    saved = m.state_dict()
    x0 = saved["collections"]["walkers"]["states"]["x"].clone()
    m.run(4)  # the model moves on; the snapshot does not
    assert torch.equal(saved["collections"]["walkers"]["states"]["x"], x0)
    assert saved["time_step"] == 3


def test_load_rejects_other_collections(cuda):
    import jaxabm_gb300 as jx
    a = jx.RandomWalkModel({"n": 500, "seed": 0}).core_model()
    a.run(2)
    b = jx.RandomWalkModel({"n": 400, "seed": 0}).core_model()
    with pytest.raises(ValueError):
        b.load_state_dict(a.state_dict())
    with pytest.raises(RuntimeError):
        jx.RandomWalkModel({"n": 10}).core_model().state_dict()
