"""One entry point for running many models as batched ensembles.

The reference runs every ensemble -- ``Model.batch_run`` (jaxabm/agentpy.py:1116-1152),
``SensitivityAnalysis.run`` (jaxabm/analysis.py:97-165), the calibrators' population and
robust evaluations (jaxabm/analysis.py:434-476) -- as a Python loop of ``model.run()``.
Here each model family that the engine batches has its own ``run_ensemble``:

* SIR (``sir.run_ensemble``): every member and step in one CUDA-graph replay;
* random walk (``randomwalk.run_ensemble``): members of one size in one launch;
* Schelling (``schelling.run_ensemble``): one thread-block cluster per member;
* opinion (``opinion.run_ensemble``): members sharing a graph as columns of one batch.

Each member's ``Results`` equal that model's own ``run()``.
"""


def _families():
    from . import opinion, randomwalk, schelling, sir
    return [(sir.SIRModel, sir.run_ensemble),
            (randomwalk.RandomWalkModel, randomwalk.run_ensemble),
            (schelling.SchellingModel, schelling.run_ensemble),
            (opinion.OpinionModel, opinion.run_ensemble)]


def run_ensemble(models):
    """One ``Results`` per model (in order), the models of each family run as one batch;
    None when some model belongs to no batchable family (or its family cannot batch it:
    Python hooks, a custom ``setup``), so the caller runs the models one by one."""
    models = list(models)
    if not models:
        return []
    fams = _families()
    groups = {}
    for k, m in enumerate(models):
        for fam, (cls, _) in enumerate(fams):
            if isinstance(m, cls):
                groups.setdefault(fam, []).append(k)
                break
        else:
            return None
    out = [None] * len(models)
    for fam, idx in groups.items():
        res = fams[fam][1]([models[k] for k in idx])
        if res is None:
            return None
        for k, r in zip(idx, res):
            out[k] = r
    return out
