"""Batching: many independent models as replicas of one device engine.

Each replica's random stream depends only on its own seed, molecule ids and
iteration count, and replicas never interact, so a replica's count trajectory
in a batch must equal the trajectory of the same model run alone — exactly
(the same kernels on the same inputs); the only way two runs could part is a
tie of two reaction times at float resolution, and the assertions allow none.
"""
import numpy as np
import pytest

from mcell_gb300 import _native
from mcell_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NSP = 3


def _models(n, seed):
    return W.replica_models(n, seed=seed, n_range=(1_000, 8_000), edge_range_um=(0.5, 1.5), levels=(2, 4))


def _alone(model, precision, seed, iters, autotune=False):
    """Trajectory of the model run by itself (a plain engine, or a one-replica batch)."""
    if not autotune:
        e = W.engine_for(model, precision, seed=seed)
        e.step(iters)
        t = e.trajectory(iters)
        e.close()
        return t
    b = _native.Batch(precision, NSP, 1, autotune=True)
    h = W.model_handle(model, precision, seed=seed)
    (r,) = b.add([h])
    h.close()
    b.step(iters)
    t = b.trajectory(r, iters)
    b.close()
    return t


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_replicas_match_models_run_alone(precision):
    ms = _models(5, seed=21)
    iters = 40
    want = [_alone(m, precision, 100 + k, iters) for k, m in enumerate(ms)]
    b = _native.Batch(precision, NSP, 8)
    hs = [W.model_handle(m, precision, seed=100 + k) for k, m in enumerate(ms)]
    ids = b.add(hs)
    for h in hs:
        h.close()
    b.step(iters)
    for k, r in enumerate(ids):
        got = b.trajectory(r, iters)
        assert np.array_equal(got, want[k]), f"replica {k}: first differing row {np.argmax((got != want[k]).any(1))}"
        assert got[-1, 2] > 0 or ms[k].bimol[0][2] < 0.01  # reactions happened
    it, steps, launches = b.stats()
    assert it == iters and launches > 0
    b.close()


def test_iteration_budget_removal_and_late_admission():
    ms = _models(4, seed=22)
    b = _native.Batch("fp32", NSP, 4)
    hs = [W.model_handle(m, "fp32", seed=200 + k) for k, m in enumerate(ms[:3])]
    ids = b.add(hs, n_iterations=[10, 0, 0])
    b.step(30)
    done, _ = b.replica_info(ids[0])
    assert done == 10
    t0 = b.trajectory(ids[0], 30)
    assert np.array_equal(t0[:10], _alone(ms[0], "fp32", 200, 10))
    assert (t0[10:] == t0[9]).all()  # frozen after its budget
    # removing one replica leaves the others undisturbed
    b.remove([ids[1]])
    b.step(10)
    assert np.array_equal(b.trajectory(ids[2], 40), _alone(ms[2], "fp32", 202, 40))
    with pytest.raises(_native.EngineError):
        b.counts(ids[1])
    # a model admitted later starts from its own iteration 0
    h = W.model_handle(ms[3], "fp32", seed=203)
    (late,) = b.add([h])
    b.step(20)
    assert np.array_equal(b.trajectory(late, 20), _alone(ms[3], "fp32", 203, 20))
    assert np.array_equal(b.trajectory(ids[2], 60), _alone(ms[2], "fp32", 202, 60))
    b.close()


def test_autotuned_batch_matches_autotuned_alone():
    ms = _models(4, seed=23)
    iters = 30
    want = [_alone(m, "fp32", 300 + k, iters, autotune=True) for k, m in enumerate(ms)]
    b = _native.Batch("fp32", NSP, 4, autotune=True)
    hs = [W.model_handle(m, "fp32", seed=300 + k) for k, m in enumerate(ms)]
    ids = b.add(hs)
    b.step(iters)
    for k, r in enumerate(ids):
        assert np.array_equal(b.trajectory(r, iters), want[k])
        _, nsub = b.replica_info(r)
        assert 1 <= nsub <= 300
    assert 1 <= b.diffuse_blocks_per_sm()
    assert b.device_bytes() > 0
    b.close()


def test_batch_molecules_stay_in_their_replica():
    ms = _models(3, seed=24)
    b = _native.Batch("fp32", NSP, 3)
    ids = b.add([W.model_handle(m, "fp32", seed=400 + k) for k, m in enumerate(ms)])
    b.step(12)
    for k, r in enumerate(ids):
        pos, sp, uid = b.molecules(r)
        lo = np.asarray(ms[k].origin)
        hi = lo + ms[k].partition_edge
        assert len(pos) == int(b.counts(r).sum())
        assert (pos >= lo).all() and (pos < hi).all()
        assert len(np.unique(uid)) == len(uid)
    b.close()


def test_batch_count_files_follow_the_replica(tmp_path):
    ms = _models(2, seed=25)
    b = _native.Batch("fp32", NSP, 2)
    ids = b.add([W.model_handle(m, "fp32", seed=800 + k) for k, m in enumerate(ms)], n_iterations=[6, 0])
    b.step(10)
    r = ids[0]  # frozen after 6 iterations: its last rows repeat
    b.write_counts(r, tmp_path / "rep", [(2, -1, "C")], n_iterations=10, every=2, fmt="gdat")
    t = b.trajectory(r, 10)
    lines = (tmp_path / "rep.gdat").read_text().splitlines()
    g = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    # a t = 0 row (no C before the first iteration), then every second iteration
    assert np.allclose(g[:, 0], [0.0, 2e-6, 4e-6, 6e-6, 8e-6, 1e-5])
    assert g[0, 1] == 0.0
    assert np.array_equal(g[1:, 1], t[[1, 3, 5, 7, 9], 2].astype(float))
    assert g[4, 1] == g[3, 1] == g[5, 1]  # frozen from iteration 6 on
    b.close()
