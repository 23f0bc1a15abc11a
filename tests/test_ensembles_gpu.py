"""Batched ensembles of the random-walk, Schelling and opinion models (``run_ensemble`` of
each family, ``batching.run_ensemble``, ``Model.batch_run``, ``SensitivityAnalysis``):
every member is checked against the oracle run of that member alone, and the batched
result equals the model's own ``run()`` (the reference's serial loop,
jaxabm/agentpy.py:1116-1152, jaxabm/analysis.py:97-165)."""

import numpy as np
import pytest

from oracle import coracle, models

pytestmark = pytest.mark.gpu


def _circ(a, b):
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    return np.minimum(d, 1.0 - d)


def test_randomwalk_ensemble_matches_oracle(cuda):
    import jaxabm_gb300 as jx
    from jaxabm_gb300 import randomwalk
    cfg = [(10_000, 0.01, 3, 60), (10_000, 0.03, 4, 60), (10_000, 0.02, 5, 60),
           (3_000, 0.01, 6, 60), (3_000, 0.05, 7, 60), (200_000, 0.01, 8, 12)]
    ms = [jx.RandomWalkModel({"n": n, "sigma": s, "steps": T}, seed=seed) for n, s, seed, T in cfg]
    runs = randomwalk.run_ensemble(ms)
    assert runs is not None and len(runs) == len(cfg)
    for (n, s, seed, T), res in zip(cfg, runs):
        ref = coracle.randomwalk_run(seed, n, T, s)
        assert _circ(res["agents.walkers.x"], ref["x"]).max() < 1e-5
        assert _circ(res["agents.walkers.y"], ref["y"]).max() < 1e-5
        np.testing.assert_allclose(np.array([res["mean_x"], res["mean_y"]]).T, ref["means"],
                                   rtol=1e-5)
        assert res["step"] == list(range(1, T + 1))
    # each member is bit-identical to its own run()
    for (n, s, seed, T), res in list(zip(cfg, runs))[::2]:
        solo = jx.RandomWalkModel({"n": n, "sigma": s, "steps": T}, seed=seed).run()
        assert np.array_equal(solo["agents.walkers.x"], res["agents.walkers.x"])
        assert solo["mean_x"] == res["mean_x"] and solo["mean_y"] == res["mean_y"]
        assert sorted(solo.keys()) == sorted(res.keys())


def test_schelling_ensemble_matches_oracle(cuda):
    import jaxabm_gb300 as jx
    from jaxabm_gb300 import schelling
    from jaxabm_gb300.schelling import initial_layout, threshold_fraction
    cfg = [(40, 40, 0.9, 0.375, 1, 25), (40, 40, 0.8, 0.5, 2, 25), (40, 40, 0.95, (2, 3), 3, 25),
           (64, 32, 0.9, 0.375, 4, 30), (256, 256, 0.9, 0.375, 5, 40)]
    ms = [jx.SchellingModel({"width": W, "height": H, "density": d, "threshold": thr,
                             "steps": T}, seed=seed) for W, H, d, thr, seed, T in cfg]
    runs = schelling.run_ensemble(ms)
    assert runs is not None
    for (W, H, d, thr, seed, T), res in zip(cfg, runs):
        pos, types = initial_layout(W, H, d, 0.5, seed)
        rng, _ = models.model_keys(seed, 1)
        ck, _ = models.keychain(rng, T, 1)
        rp, rstats = coracle.schelling_run(pos, types, W, H, ck.reshape(T, 2),
                                           threshold_fraction(thr))
        assert np.array_equal(np.array([res["unhappy"], res["moved"]]).T, rstats), seed
        assert np.array_equal(res["agents.agents.position"], rp), seed
    solo = ms[1].__class__(dict(ms[1].p), seed=ms[1].seed).run()
    assert sorted(solo.keys()) == sorted(runs[1].keys())
    assert np.array_equal(solo["agents.agents.position"], runs[1]["agents.agents.position"])


def test_opinion_ensemble_matches_oracle(cuda):
    """Members sharing a graph run as columns of one batch: final opinions equal the float32
    oracle bit for bit and the per-step moments equal the solo run's exactly."""
    import jaxabm_gb300 as jx
    from jaxabm_gb300 import opinion
    from jaxabm_gb300.opinion import initial_opinions
    from oracle import workloads
    n, T = 4096, 30
    cfg = [(0.3, 0.2, 0.02, 11), (0.25, 0.15, 0.025, 12), (0.35, 0.22, 0.018, 13),
           (0.3, 0.2, 0.02, 14), (0.28, 0.19, 0.021, 15)]
    ms = [jx.OpinionModel({"n": n, "steps": T, "graph_seed": 7, "mu": mu, "eps": e, "tau": t},
                          seed=s) for mu, e, t, s in cfg]
    ms.append(jx.OpinionModel({"n": 2048, "steps": T, "mu": 0.3}, seed=21))  # its own graph
    runs = opinion.run_ensemble(ms)
    rp, col = workloads.random_regular(n, 16, 7)
    for (mu, e, t, s), res in zip(cfg, runs):
        o0 = initial_opinions(n, s).cpu().numpy()[:, None]
        ref = coracle.opinion_run_f32(o0, rp, col, [mu], [e], [t], T)[:, 0]
        assert np.array_equal(res["agents.people.opinion"].view(np.uint32),
                              ref.view(np.uint32)), s
        m = coracle.opinion_moments_f64(ref[:, None].astype(np.float64))[0]
        np.testing.assert_allclose([res[f"m{q}"][-1] for q in range(1, 5)], m, rtol=1e-12)
    rp2, col2 = workloads.random_regular(2048, 16, 21)
    ref2 = coracle.opinion_run_f32(initial_opinions(2048, 21).cpu().numpy()[:, None], rp2, col2,
                                   [0.3], [0.2], [0.02], T)[:, 0]
    assert np.array_equal(runs[-1]["agents.people.opinion"], ref2)
    solo = ms[2].run()
    assert np.array_equal(solo["agents.people.opinion"], runs[2]["agents.people.opinion"])
    for q in range(1, 5):
        assert solo[f"m{q}"] == runs[2][f"m{q}"]


def test_batching_dispatch_and_batch_run(cuda):
    """batching.run_ensemble takes models of several families at once; Model.batch_run of a
    random-walk model goes through it and equals the serial runs; a model with a Python
    hook is not batched."""
    import jaxabm_gb300 as jx
    from jaxabm_gb300 import batching
    mix = [jx.RandomWalkModel({"n": 2000, "steps": 10}, seed=1),
           jx.SIRModel({"n": 3000, "steps": 20, "m": 3}, seed=2),
           jx.SchellingModel({"width": 20, "height": 20, "steps": 10}, seed=3),
           jx.RandomWalkModel({"n": 2000, "steps": 10, "sigma": 0.02}, seed=4)]
    runs = batching.run_ensemble(mix)
    for m, res in zip(mix, runs):
        solo = m.__class__(dict(m.p), seed=m.seed).run()
        for k in solo.keys():
            assert np.array_equal(np.asarray(solo[k]), np.asarray(res[k])), (type(m), k)
    base = jx.RandomWalkModel({"n": 1500, "steps": 8}, seed=9)
    res = base.batch_run({"sigma": [0.01, 0.04]}, repetitions=2)
    for (sigma,), reps in res.items():
        for r, got in enumerate(reps):
            ref = jx.RandomWalkModel({"n": 1500, "steps": 8, "sigma": sigma}, seed=9 + r).run()
            assert got["mean_x"] == ref["mean_x"]

    class Hooked(jx.RandomWalkModel):
        def step(self):
            pass
    assert batching.run_ensemble([Hooked({"n": 100, "steps": 2}, seed=0)]) is None


def test_sensitivity_analysis_batches_opinion_models(cuda):
    import jaxabm_gb300 as jx

    def factory(params=None, config=None):
        return jx.OpinionModel(dict(n=2048, steps=15, graph_seed=3, **params), seed=config.seed)
    sa = jx.SensitivityAnalysis(factory, {"mu": (0.2, 0.4), "eps": (0.1, 0.3)}, ["m2"],
                                num_samples=12, seed=1)
    res = sa.run(verbose=False)
    assert sa.batched
    host = sa.samples.cpu().numpy()
    for i in (0, 5, 11):
        ref = factory(params={"mu": float(host[i, 0]), "eps": float(host[i, 1])},
                      config=jx.ModelConfig(seed=1000 + i)).run()
        assert float(res["m2"][i]) == pytest.approx(ref["m2"][-1], rel=1e-6)
