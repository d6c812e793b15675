"""Serving: requests arrive while others run, are continuously batched, and each
result (the species-count trajectory) must equal the same model run alone —
exactly, since a request's random stream depends only on its own seed,
molecule ids and iteration count."""
import time

import numpy as np
import pytest

from mcell_gb300 import _native
from mcell_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NSP = 3


def _models(n, seed):
    return W.replica_models(n, seed=seed, n_range=(1_000, 6_000), edge_range_um=(0.5, 1.2), levels=(2, 3))


def _alone(model, seed, iters):
    e = W.engine_for(model, "fp32", seed=seed)
    e.step(iters)
    t = e.trajectory(iters)
    e.close()
    return t


def test_served_results_match_models_run_alone():
    ms = _models(6, seed=31)
    iters = [30, 75, 20, 50, 64, 33]
    srv = _native.Server("fp32", NSP, max_slots=3, autotune=False)  # fewer slots than requests: some queue
    tickets = []
    for k, m in enumerate(ms):
        h = W.model_handle(m, "fp32", seed=500 + k)
        tickets.append(srv.submit(h, iters[k]))
        h.close()  # the server copied the model
        time.sleep(0.005)  # later requests arrive while earlier ones run
    for k, t in enumerate(tickets):
        assert srv.wait(t, 300) == "done"
        final, traj = srv.result(t)
        want = _alone(ms[k], 500 + k, iters[k])
        assert traj.shape == want.shape
        assert np.array_equal(traj, want), f"request {k}"
        assert np.array_equal(final, want[-1])
        state, seconds = srv.poll(t)
        assert state == "done" and seconds > 0
    st = srv.stats()
    assert st["completed"] == 6 and st["failed"] == 0 and st["mol_steps"] > 0
    srv.close()


def test_budget_admission_and_cancel():
    ms = _models(4, seed=32)
    budget = 6 << 20
    srv = _native.Server("fp32", NSP, max_slots=1, hbm_budget_bytes=budget, autotune=False)
    hs = [W.model_handle(m, "fp32", seed=600 + k) for k, m in enumerate(ms)]
    t_long = srv.submit(hs[0], 5000)
    t_mid = srv.submit(hs[1], 40)
    t_drop = srv.submit(hs[2], 40)
    srv.cancel(t_drop)  # still queued behind the long one (one slot)
    assert srv.poll(t_drop)[0] == "cancelled"
    for _ in range(200):
        if srv.poll(t_long)[0] == "running":
            break
        time.sleep(0.01)
    assert srv.poll(t_mid)[0] == "queued"
    assert srv.stats()["reserved_bytes"] <= budget
    srv.cancel(t_long)  # stops at the end of its current block
    assert srv.wait(t_long, 120) == "cancelled"
    assert srv.wait(t_mid, 300) == "done"
    assert np.array_equal(srv.result(t_mid)[1], _alone(ms[1], 601, 40))
    with pytest.raises(_native.EngineError):
        srv.result(t_drop)
    srv.release(t_drop)
    with pytest.raises(_native.EngineError):
        srv.poll(t_drop)
    tiny = _native.Server("fp32", NSP, max_slots=4, hbm_budget_bytes=1024, autotune=False)
    with pytest.raises(_native.EngineError) as ei:
        tiny.submit(hs[3], 10)  # larger than the whole budget
    assert ei.value.code == -3
    tiny.close()
    srv.close()
