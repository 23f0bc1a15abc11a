"""Continuous-batching server: every request's result is identical alone and in the mix,
admission respects slots/tiles/memory, and requests arriving while others run overlap."""

import numpy as np
import pytest
import torch

from oracle import coracle, models

pytestmark = pytest.mark.gpu


def _requests(k, seed0=100, steps=60):
    from jaxabm_gb300 import sir
    from jaxabm_gb300.serving import Request
    rs = np.random.RandomState(seed0)
    reqs = []
    for i in range(k):
        n = int(rs.randint(300, 20_000))
        s = seed0 + i
        rp, col = sir.barabasi_albert(n, 4, s)
        st = sir.initial_states(n, 0.005, s)
        reqs.append(Request(i, rp, col, st, float(rs.uniform(0.02, 0.2)),
                            float(rs.uniform(0.05, 0.3)), s, steps, keep_state=True))
    return reqs


@pytest.mark.parametrize("path", ["resident", "grid"])
def test_results_identical_alone_and_in_mix(cuda, path):
    from jaxabm_gb300.serving import SIRServer
    reqs = _requests(24)
    # mix: all submitted at once into a small server (forces queueing + slot reuse)
    srv = SIRServer(max_slots=6, max_tiles=256, steps_per_tick=7, path=path)
    assert srv.resident == (path == "resident")
    for r in reqs:
        srv.submit(r)
    srv.drain()
    srv.check()
    assert len(srv.completed) == len(reqs)
    mixed = {r.rid: (r.counts.numpy().copy(), r.final_state.numpy().copy()) for r in srv.completed}
    # alone: each request by itself through a fresh server
    for r in _requests(24)[::5]:
        solo = SIRServer(max_slots=1, max_tiles=128, steps_per_tick=13,
                         path="grid" if path == "resident" else "resident")
        solo.submit(r)
        solo.drain()
        c, fs = mixed[r.rid]
        assert np.array_equal(solo.completed[0].counts.numpy(), c)
        assert np.array_equal(solo.completed[0].final_state.numpy(), fs)
    # and against the oracle
    for r in _requests(24)[:4]:
        rng, _ = models.model_keys(r.seed, 1)
        ref_st, ref_counts, _ = coracle.sir_run(r.row_ptr, r.col, r.state, rng, r.steps,
                                                r.beta, r.gamma)
        c, fs = mixed[r.rid]
        assert np.array_equal(c, ref_counts)
        assert np.array_equal(fs, ref_st)


def test_overlap_and_slot_limit(cuda):
    from jaxabm_gb300.serving import SIRServer
    reqs = _requests(10, seed0=7, steps=40)
    srv = SIRServer(max_slots=3, max_tiles=512, steps_per_tick=4)
    for r in reqs:
        srv.submit(r)
    max_active = 0
    while not srv.idle():
        srv.tick()
        max_active = max(max_active, len(srv.active))
        assert len(srv.active) <= 3
    assert max_active == 3  # several requests were on the device together
    assert len(srv.completed) == 10
    adm = sorted(r.admitted for r in srv.completed)
    fin = sorted(r.finished for r in srv.completed)
    assert adm[3] < fin[-1]  # later requests were admitted while others were running


def test_admission_by_free_memory(cuda, monkeypatch):
    from jaxabm_gb300.serving import SIRServer
    reqs = _requests(3, seed0=11, steps=10)
    srv = SIRServer(max_slots=4, max_tiles=256, steps_per_tick=5, reserve_bytes=0)
    # pretend the device has room for exactly one request
    budget = reqs[0].device_bytes() + 1
    monkeypatch.setattr(SIRServer, "free_bytes",
                        staticmethod(lambda: budget - sum(r.device_bytes() for r in srv.active.values())))
    for r in reqs:
        srv.submit(r)
    srv.tick()
    assert len(srv.active) == 1 and len(srv.queue) == 2
    srv.drain()
    assert len(srv.completed) == 3


def test_resident_server_rejects_oversize_request(cuda):
    from jaxabm_gb300 import sir
    from jaxabm_gb300.serving import Request, SIRServer
    srv = SIRServer(max_slots=2, max_tiles=64, steps_per_tick=3, path="resident",
                    max_request_agents=1000)
    rp, col = sir.barabasi_albert(1500, 4, 1)
    with pytest.raises(ValueError):
        srv.submit(Request(0, rp, col, sir.initial_states(1500, 0.01, 1), 0.1, 0.1, 1, 5))


@pytest.mark.parametrize("path", ["resident", "grid"])
def test_bad_request_reports_its_error_and_others_finish(cuda, path):
    """A request whose network has a column outside its agents, and one with a compartment
    outside 0..2, each come back with an AbmError naming the fault; the other requests of
    the same admission group finish with the oracle's results."""
    from jaxabm_gb300 import _lib
    from jaxabm_gb300.serving import SIRServer
    reqs = _requests(6, seed0=300, steps=30)
    bad_col = reqs[2]
    bad_col.col = bad_col.col.copy()
    bad_col.col[3] = bad_col.n + 5
    bad_st = reqs[4]
    bad_st.state = bad_st.state.copy()
    bad_st.state[0] = 9
    srv = SIRServer(max_slots=8, max_tiles=256, steps_per_tick=10, path=path)
    for r in reqs:
        srv.submit(r)
    srv.drain()
    done = {r.rid: r for r in srv.completed}
    assert done[2].error is not None and done[2].error.status == _lib.ABM_ERR_BOUNDS
    assert "CSR column" in str(done[2].error)
    assert done[4].error is not None and "compartment" in str(done[4].error)
    for rid in (0, 1, 3, 5):
        r = done[rid]
        assert r.error is None
        rng, _ = models.model_keys(r.seed, 1)
        _, ref_counts, _ = coracle.sir_run(r.row_ptr, r.col, r.state, rng, r.steps, r.beta,
                                           r.gamma)
        assert np.array_equal(r.counts.numpy(), ref_counts), rid


@pytest.mark.parametrize("path", ["resident", "grid"])
def test_cancel_queued_and_running_requests(cuda, path):
    """cancel() drops a queued request and stops a running one between ticks; its slot is
    reused, and every other request still equals the oracle."""
    from jaxabm_gb300.serving import SIRServer
    reqs = _requests(8, seed0=400, steps=80)
    srv = SIRServer(max_slots=3, max_tiles=64, steps_per_tick=5, path=path)
    for r in reqs:
        srv.submit(r)
    srv.tick()
    srv.tick()
    running = next(iter(srv.active.values())).rid
    queued = srv.queue[-1].rid
    assert srv.cancel(running) and srv.cancel(queued)
    assert not srv.cancel(10_000)
    srv.drain()
    assert sorted(r.rid for r in srv.cancelled) == sorted([running, queued])
    assert all(r.cancelled for r in srv.cancelled)
    finished = {r.rid: r for r in srv.completed}
    assert set(finished) == {r.rid for r in reqs} - {running, queued}
    for rid, r in finished.items():
        rng, _ = models.model_keys(r.seed, 1)
        ref_st, ref_counts, _ = coracle.sir_run(r.row_ptr, r.col, r.state, rng, r.steps, r.beta,
                                                r.gamma)
        assert np.array_equal(r.counts.numpy(), ref_counts), rid
        assert np.array_equal(r.final_state.numpy(), ref_st), rid


@pytest.mark.parametrize("path", ["resident", "grid"])
def test_page_locked_requests_take_the_gather_copies(cuda, path):
    """Requests whose arrays are page-locked tensors are admitted and retired through the
    one-launch gather copy (abm_copy_segments_kernel); numpy requests in the same server go
    through per-array copies.  Every result equals its oracle run either way."""
    from jaxabm_gb300.serving import Request, SIRServer
    base = _requests(10, seed0=700, steps=40)
    reqs = []
    for r in base:
        if r.rid % 2 == 0:  # every other request page-locked
            r = Request(r.rid, torch.from_numpy(np.asarray(r.row_ptr)).pin_memory(),
                        torch.from_numpy(np.asarray(r.col)).pin_memory(),
                        torch.from_numpy(np.asarray(r.state)).pin_memory(),
                        r.beta, r.gamma, r.seed, r.steps)
            assert r._pinned
        else:
            assert not r._pinned
        reqs.append(r)
    srv = SIRServer(max_slots=4, max_tiles=128, steps_per_tick=9, path=path)
    for r in reqs[:5]:
        srv.submit(r)
    srv.tick()
    for r in reqs[5:]:
        srv.submit(r)
    srv.drain()
    srv.check()
    assert len(srv.completed) == len(reqs)
    for r in srv.completed:
        rng, _ = models.model_keys(r.seed, 1)
        _, ref_counts, _ = coracle.sir_run(np.asarray(r.row_ptr), np.asarray(r.col),
                                           np.asarray(r.state), rng, r.steps, r.beta, r.gamma)
        assert np.array_equal(r.counts.numpy(), ref_counts), r.rid
