"""Differentiable bounded-confidence opinion model and its calibration gradient.

Model (per step, every agent reads the pre-step opinions)::

    o_i += mu * mean_j sigmoid((eps - |o_j - o_i|) / tau) * (o_j - o_i)

on a symmetric network (``Network``, CSR).  ``OpinionBatch`` evaluates B parameter sets at
once on one graph (opinions interleaved ``[N][B]``), stores a checkpoint every ``k`` steps
on the forward pass, and computes d loss / d (mu, eps, tau) with the hand-written reverse
sweep: each segment of ``k`` steps is recomputed from its checkpoint, then the adjoint
kernel walks it backwards.  ``OpinionLoss`` wraps this as a ``torch.autograd.Function``.

The reference calibrates by ``jit(grad(loss_fn))`` through its whole Python run loop
(jaxabm/analysis.py:494-522, ``ModelCalibrator._calibrate_gradient``); the loss here is the
mean squared error of the first four raw opinion moments at step T against a target.
"""

import numpy as np
import torch

from . import _dev
from . import _lib
from . import random as jrandom
from .agentpy import Agent, Model, Network
from .registry import StepKernel, register_step


def _pow2_at_least(b, lo=4):
    p = lo
    while p < b:
        p *= 2
    return p


def initial_opinions(n, seed=0):
    """o_i = uniform(split(init_key, n)[i]) with the collection init key of
    ``Model.initialize`` for ``seed`` (one collection)."""
    keys = jrandom.split(jrandom.PRNGKey(seed), 2)
    agent_keys = jrandom.split(keys[1].contiguous(), n)
    return jrandom.uniform(agent_keys)


class OpinionBatch:
    """B opinion models (one parameter set each) on one graph.

    Args:
        row_ptr, col: symmetric CSR (host arrays or device tensors)
        o0: initial opinions, float32[N] (shared) or [N, B]
        mu, eps, tau: float32[B]
    """

    def __init__(self, row_ptr, col, o0, mu, eps, tau):
        dev = _dev.device()
        self.rp = torch.as_tensor(np.asarray(row_ptr) if not isinstance(row_ptr, torch.Tensor)
                                  else row_ptr, dtype=torch.int32).to(dev).contiguous()
        self.col = torch.as_tensor(np.asarray(col) if not isinstance(col, torch.Tensor)
                                   else col, dtype=torch.int32).to(dev).contiguous()
        self.n = self.rp.numel() - 1
        mu = torch.as_tensor(mu, dtype=torch.float32).reshape(-1)
        self.B_user = mu.numel()
        self.B = _pow2_at_least(self.B_user)
        if self.B > 128:
            raise ValueError("at most 128 instances per batch")
        self.set_params(mu, eps, tau)
        o0 = torch.as_tensor(o0, dtype=torch.float32).to(dev)
        if o0.dim() == 1:
            o0 = o0[:, None].expand(self.n, self.B_user)
        self.o0 = self._pad_cols(o0).contiguous()
        self.o = self.o0.clone()
        self.tmp = torch.empty_like(self.o)
        self.ckpts = None
        self.inv_deg = None  # 1 / degree per node, built by the first backward
        self.ckpt_every = None
        self.steps_done = 0

    def _pad_cols(self, x):
        if x.shape[-1] == self.B:
            return x.contiguous()
        pad = x[..., :1].expand(*x.shape[:-1], self.B - x.shape[-1])
        return torch.cat([x, pad], dim=-1).contiguous()

    def set_params(self, mu, eps, tau):
        dev = _dev.device()
        vals = [torch.as_tensor(v, dtype=torch.float32).reshape(-1).to(dev) for v in (mu, eps, tau)]
        self.mu, self.eps, self.tau = (self._pad_cols(v[None])[0] for v in vals)

    def reset(self):
        self.o.copy_(self.o0)
        self.steps_done = 0

    def forward(self, steps, ckpt_every=None):
        """Run ``steps`` steps from the initial state; keep checkpoints every
        ``ckpt_every`` steps for :meth:`backward`."""
        self.reset()
        ck = None
        if ckpt_every:
            nck = (steps + ckpt_every - 1) // ckpt_every
            ck = torch.empty((nck, self.n, self.B), dtype=torch.float32, device=self.o.device)
        _lib.call("abm_opinion_run", _dev.ptr(self.o), _dev.ptr(self.tmp), _dev.ptr(self.rp),
                  _dev.ptr(self.col), self.n, self.B, _dev.ptr(self.mu), _dev.ptr(self.eps),
                  _dev.ptr(self.tau), int(steps), int(ckpt_every or 0),
                  _dev.ptr(ck) if ck is not None else None, _dev.stream_handle())
        self.ckpts, self.ckpt_every, self.steps_done = ck, ckpt_every, steps
        return self.o

    def forward_with_moments(self, steps):
        """``steps`` forward steps from the initial state (no checkpoints), with the raw
        moments after every step: float64[steps, B_user, 4]."""
        self.reset()
        dev = self.o.device
        rows = torch.empty((steps, self.B, 4), dtype=torch.float64, device=dev)
        ws = _dev.workspace(_lib.load().abm_opinion_moments_workspace_bytes(self.n, self.B))
        cur, nxt = self.o, self.tmp
        for t in range(steps):
            _lib.call("abm_opinion_step", _dev.ptr(cur), _dev.ptr(nxt), _dev.ptr(self.rp),
                      _dev.ptr(self.col), self.n, self.B, _dev.ptr(self.mu), _dev.ptr(self.eps),
                      _dev.ptr(self.tau), _dev.stream_handle())
            _lib.call("abm_opinion_moments", _dev.ptr(nxt), self.n, self.B, _dev.ptr(rows[t]),
                      _dev.ptr(ws), ws.numel(), _dev.stream_handle())
            cur, nxt = nxt, cur
        if cur is not self.o:
            self.o.copy_(cur)
        self.ckpts, self.ckpt_every, self.steps_done = None, None, steps
        return rows[:, :self.B_user]

    def moments(self, o=None):
        """Raw moments float64[B_user, 4] of the current (or given) state."""
        o = self.o if o is None else o
        out = torch.empty((self.B, 4), dtype=torch.float64, device=o.device)
        ws = _dev.workspace(_lib.load().abm_opinion_moments_workspace_bytes(self.n, self.B))
        _lib.call("abm_opinion_moments", _dev.ptr(o), self.n, self.B, _dev.ptr(out), _dev.ptr(ws),
                  ws.numel(), _dev.stream_handle())
        return out[:self.B_user]

    @staticmethod
    def loss_of(moments, target):
        t = torch.as_tensor(target, dtype=torch.float64, device=moments.device).reshape(-1, 4)
        return 0.25 * ((moments - t) ** 2).sum(dim=1)

    def backward(self, target, grad_loss=None):
        """d loss_b / d (mu_b, eps_b, tau_b) -> float64[B_user, 3] after :meth:`forward`
        with checkpoints; ``grad_loss`` (float64[B_user]) scales each instance."""
        dev = self.o.device
        m = self.moments()
        t = torch.as_tensor(target, dtype=torch.float64, device=dev).reshape(-1, 4)
        dldm = 0.5 * (m - t)
        if grad_loss is not None:
            dldm = dldm * torch.as_tensor(grad_loss, dtype=torch.float64, device=dev).reshape(-1, 1)
        return self.backward_moments(dldm)

    def backward_moments(self, dldm):
        """Vector-Jacobian product of the final raw moments: given d loss_b / d m_k
        (float64[B_user, 4]) after :meth:`forward` with checkpoints, returns
        d loss_b / d (mu_b, eps_b, tau_b) as float64[B_user, 3] by the reverse sweep."""
        if self.ckpts is None:
            raise RuntimeError("forward(steps, ckpt_every) must run first")
        dev = self.o.device
        T, k = self.steps_done, self.ckpt_every
        dldm = torch.as_tensor(dldm, dtype=torch.float64, device=dev).reshape(-1, 4)
        dl = torch.zeros((self.B, 4), dtype=torch.float64, device=dev)
        dl[:self.B_user] = dldm
        lam = torch.empty_like(self.o)
        lam2 = torch.empty_like(self.o)
        _lib.call("abm_opinion_adjoint_init", _dev.ptr(self.o), self.n, self.B, _dev.ptr(dl),
                  _dev.ptr(lam), _dev.stream_handle())
        gws = torch.zeros(_lib.load().abm_opinion_grad_workspace_bytes(self.n, self.B) // 8,
                          dtype=torch.float64, device=dev)
        seg = torch.empty((k - 1, self.n, self.B), dtype=torch.float32, device=dev)
        if self.inv_deg is None:
            self.inv_deg = torch.empty(self.n, dtype=torch.float32, device=dev)
            _lib.call("abm_opinion_inv_degree", _dev.ptr(self.rp), self.n, _dev.ptr(self.inv_deg),
                      _dev.stream_handle())
        nseg = self.ckpts.shape[0]
        for s in range(nseg - 1, -1, -1):
            t0 = s * k
            length = min(k, T - t0)
            # recompute o^{t0+1} .. o^{t0+length-1} from the checkpoint o^{t0}
            states = [self.ckpts[s]] + [seg[q] for q in range(length - 1)]
            for q in range(1, length):
                _lib.call("abm_opinion_step", _dev.ptr(states[q - 1]), _dev.ptr(states[q]),
                          _dev.ptr(self.rp), _dev.ptr(self.col), self.n, self.B,
                          _dev.ptr(self.mu), _dev.ptr(self.eps), _dev.ptr(self.tau),
                          _dev.stream_handle())
            for q in range(length - 1, -1, -1):
                _lib.call("abm_opinion_adjoint_step", _dev.ptr(states[q]), _dev.ptr(lam),
                          _dev.ptr(lam2), _dev.ptr(self.rp), _dev.ptr(self.col),
                          _dev.ptr(self.inv_deg), self.n, self.B, _dev.ptr(self.mu),
                          _dev.ptr(self.eps), _dev.ptr(self.tau), _dev.ptr(gws), gws.numel() * 8,
                          _dev.stream_handle())
                lam, lam2 = lam2, lam
        grads = torch.empty((self.B, 3), dtype=torch.float64, device=dev)
        _lib.call("abm_opinion_grad_reduce", _dev.ptr(gws), self.n, self.B, _dev.ptr(grads),
                  _dev.stream_handle())
        return grads[:self.B_user]


class OpinionLoss(torch.autograd.Function):
    """loss[b] = 0.25 * sum_k (m_k(T; mu_b, eps_b, tau_b) - target_k)^2 with the adjoint
    kernel as its backward.  ``OpinionLoss.apply(mu, eps, tau, batch, target, steps, k)``."""

    @staticmethod
    def forward(ctx, mu, eps, tau, batch, target, steps, ckpt_every):
        batch.set_params(mu.detach(), eps.detach(), tau.detach())
        batch.forward(int(steps), int(ckpt_every))
        m = batch.moments()
        ctx.batch, ctx.target = batch, target
        return OpinionBatch.loss_of(m, target).to(mu.dtype)

    @staticmethod
    def backward(ctx, grad_loss):
        g = ctx.batch.backward(ctx.target, grad_loss.detach().to(torch.float64))
        gm, ge, gt = (g[:, i].to(grad_loss.dtype) for i in range(3))
        return gm, ge, gt, None, None, None, None


# ---- single-model API --------------------------------------------------------------------

class OpinionKernel(StepKernel):
    """Registered step of ``OpinionAgent``.  Metrics ``m1``..``m4``: the raw moments
    mean_i o_i^k of the opinions after each step (float64 accumulation)."""
    name = "opinion"
    attributes = ("opinion",)
    metrics = ("m1", "m2", "m3", "m4")
    params = {"mu": 0.3, "eps": 0.2, "tau": 0.02}

    def init(self, n, init_key, params, env):
        agent_keys = jrandom.split(init_key.contiguous(), n)
        return {"opinion": jrandom.uniform(agent_keys)}

    def run(self, states, coll_keys, params, env):
        steps = coll_keys.reshape(-1, 2).shape[0]
        b = OpinionBatch(env["network_row_ptr"], env["network_col"], states["opinion"],
                         [params["mu"]], [params["eps"]], [params["tau"]])
        rows = b.forward_with_moments(steps)
        return {"opinion": b.o[:, 0].contiguous()}, rows[:, 0, :]

    def step(self, states, coll_key, params, env):
        new, rows = self.run(states, coll_key.reshape(1, 2), params, env)
        return new, rows[0]


class OpinionAgent(Agent):
    """Bounded-confidence opinion agent on a Network (registered: ``abm_opinion_*``)."""

    def setup(self, key=None):
        return {"opinion": jrandom.uniform(key)}


register_step(OpinionAgent, OpinionKernel())


class OpinionModel(Model):
    """Parameters: ``n`` (2^18), ``degree`` (16, random regular graph), ``mu``, ``eps``,
    ``tau``, ``steps`` (200), ``seed`` (initial opinions), ``graph_seed`` (the graph;
    default ``seed``).  Metrics ``m1``..``m4``: raw opinion moments after each step.

    Differentiable: :meth:`final_metrics_vjp` gives the moments after ``steps`` steps and
    their vector-Jacobian product with respect to ``mu``, ``eps``, ``tau`` (the hand-written
    adjoint), which ``ModelCalibrator(method="adam" | "sgd")`` uses in place of the
    reference's ``jit(grad(loss))`` through ``model.run`` (jaxabm/analysis.py:489-531)."""

    DIFFERENTIABLE = ("mu", "eps", "tau")

    def setup(self):
        from .sir import random_regular
        n = int(self.p.get("n", 1 << 18))
        rp, col = random_regular(n, int(self.p.get("degree", 16)),
                                 int(self.p.get("graph_seed", self.seed)))
        self.network = Network(self)
        self.network.from_csr(rp, col)
        self.agents = self.add_agents(n, OpinionAgent, name="people",
                                      mu=float(self.p.get("mu", 0.3)),
                                      eps=float(self.p.get("eps", 0.2)),
                                      tau=float(self.p.get("tau", 0.02)))


    def final_metrics_vjp(self, names, steps=None, ckpt_every=20):
        """(metrics, vjp) of a run of ``steps`` steps (default: the model's): ``metrics``
        maps ``m1``..``m4`` to the raw moments after the last step (the values ``run``
        records last); ``vjp(dl_dmetrics)`` maps d loss / d metric (a dict, missing metrics
        0) to d loss / d parameter for ``names`` (a subset of mu, eps, tau), by the adjoint
        with a checkpoint every ``ckpt_every`` steps."""
        bad = [k for k in names if k not in self.DIFFERENTIABLE]
        if bad:
            raise ValueError(f"parameters {bad} are not differentiable in OpinionModel "
                             f"(differentiable: {', '.join(self.DIFFERENTIABLE)})")
        if self._hooks() != (None, None):
            raise ValueError("a model with Python step hooks has no adjoint")
        from .core import ModelConfig
        from .model import Model as JaxModel
        steps = int(self.steps if steps is None else steps)
        # set up and initialise exactly as run() does (same graph, key chain and states)
        self.setup()
        jm = JaxModel(params=self.p, config=ModelConfig(steps=steps, seed=self.seed))
        for name, agent_list in self._agent_lists.items():
            jm.add_agent_collection(name, agent_list.collection)
        for name, value in self.env.state.items():
            jm.add_env_state(name, value)
        jm.initialize()
        if len(jm.agent_collections) != 1:
            raise ValueError("the adjoint covers models with one agent collection")
        coll = next(iter(jm.agent_collections.values()))
        if not isinstance(coll.kernel, OpinionKernel):
            raise ValueError("the adjoint covers OpinionAgent collections")
        par, env = coll.params, coll._env
        b = OpinionBatch(env["network_row_ptr"], env["network_col"], coll.states["opinion"],
                         [par["mu"]], [par["eps"]], [par["tau"]])
        b.forward(steps, max(1, min(int(ckpt_every), steps)))
        m = b.moments()[0].cpu().numpy()
        metrics = {f"m{k + 1}": float(m[k]) for k in range(4)}

        def vjp(dl_dmetrics):
            d = np.array([[float(dl_dmetrics.get(f"m{k + 1}", 0.0)) for k in range(4)]])
            g = b.backward_moments(d)[0].cpu().numpy()
            return {k: float(g[self.DIFFERENTIABLE.index(k)]) for k in names}
        return metrics, vjp


def calibration_params(count=64, base=(0.3, 0.2, 0.02), spread=0.2, seed=0):
    """``count`` parameter sets base * (1 + spread * U[-1, 1]) (RandomState(seed)); set 0 is
    the base point."""
    u = np.random.RandomState(seed).uniform(-1.0, 1.0, size=(count, 3))
    u[0] = 0.0
    p = np.asarray(base)[None, :] * (1.0 + spread * u)
    return p.astype(np.float32)


HIDDEN_PARAMS = (0.25, 0.15, 0.025)


def ensemble_member(model):
    """``(n, degree, graph_seed, mu, eps, tau, seed, steps)`` of an ``OpinionModel`` that
    can run as a batch member, else None."""
    if not isinstance(model, OpinionModel) or model._hooks() != (None, None) \
            or type(model).setup is not OpinionModel.setup:
        return None
    p = model.p
    return (int(p.get("n", 1 << 18)), int(p.get("degree", 16)),
            int(p.get("graph_seed", model.seed)), float(p.get("mu", 0.3)),
            float(p.get("eps", 0.2)), float(p.get("tau", 0.02)), int(model.seed),
            int(model.steps))


def run_ensemble(models):
    """Opinion models that share a graph (same ``n``, ``degree`` and ``graph_seed``) and step
    count run as the columns of one ``OpinionBatch`` (up to 128 per batch): each column
    has its own parameters and initial opinions, and equals its model's own ``run()``
    (keys ``step``, ``m1``..``m4``, ``agents.people.opinion``) bit for bit.  Returns None
    unless every model is a batchable ``OpinionModel``."""
    from .agentpy import Results
    from .sir import random_regular
    specs = [ensemble_member(m) for m in models]
    if any(s is None for s in specs):
        return None
    out = [None] * len(models)
    groups = {}
    for k, s in enumerate(specs):
        groups.setdefault((s[0], s[1], s[2], s[7]), []).append(k)
    for (n, degree, graph_seed, steps), idx in groups.items():
        rp, col = random_regular(n, degree, graph_seed)
        for c0 in range(0, len(idx), 128):
            part = idx[c0:c0 + 128]
            o0 = torch.stack([initial_opinions(n, specs[k][6]) for k in part], dim=1)
            b = OpinionBatch(rp, col, o0, [specs[k][3] for k in part],
                             [specs[k][4] for k in part], [specs[k][5] for k in part])
            rows = b.forward_with_moments(steps).cpu().numpy() if steps > 0 else None
            final = b.o[:, :len(part)].cpu().numpy()
            for j, k in enumerate(part):
                data = {"agents.people.opinion": final[:, j].copy()}
                if steps > 0:
                    data = {"step": list(range(1, steps + 1)),
                            **{f"m{q + 1}": rows[:, j, q].tolist() for q in range(4)}, **data}
                out[k] = Results(data)
    return out


def main(argv=None):
    """``python -m jaxabm_gb300.opinion``: times one calibration batch -- the forward with a
    checkpoint every ``--every`` steps, then the reverse sweep -- on a random
    ``--degree``-regular graph of ``--n`` nodes with ``--instances`` parameter sets, and
    prints one JSON line per repetition (CUDA events on the current stream)."""
    import argparse
    import json

    from . import _build
    from .sir import random_regular
    ap = argparse.ArgumentParser(prog="python -m jaxabm_gb300.opinion")
    ap.add_argument("--n", type=int, default=1 << 18)
    ap.add_argument("--degree", type=int, default=16)
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args(argv)
    _build.build()
    rp, col = random_regular(args.n, args.degree, 0)
    p = calibration_params(args.instances)
    b = OpinionBatch(rp, col, initial_opinions(args.n, 0), p[:, 0], p[:, 1], p[:, 2])
    target = np.array([0.5, 0.3, 0.2, 0.15])
    for rep in range(args.reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        b.forward(args.steps, args.every)
        ev[1].record()
        g = b.backward(target)
        ev[2].record()
        ev[2].synchronize()
        print(json.dumps({"rep": rep, "n": args.n, "instances": args.instances,
                          "steps": args.steps, "every": args.every,
                          "ms_forward": ev[0].elapsed_time(ev[1]),
                          "ms_reverse": ev[1].elapsed_time(ev[2]),
                          "grad_sum": float(g.sum())}), flush=True)


if __name__ == "__main__":
    main()
