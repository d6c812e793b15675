"""Out-of-memory paths, run without exhausting HBM: a test hook makes one device
allocation fail (mcg_inject_device_alloc_failure). Every call that meets it returns
MCG_ERR_CUDA with the CUDA message; nothing leaks; a failed resize leaves the engine
with its molecules and capacity as they were; and afterwards the same model runs to
the same result as if nothing had happened."""
import numpy as np
import pytest

from mcell_gb300 import _native
from mcell_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ITERS = 8


def _run(m, seed=3):
    h = W.model_handle(m, "fp32", seed=seed)
    try:
        h.prepare()
        h.step(ITERS)
        return h.trajectory(ITERS)
    finally:
        h.close()


def test_allocation_failure_at_every_point_of_a_run():
    m = W.closed_cube(n_per_species=2000)
    base = _run(m)
    failed = 0
    for after in range(0, 40):
        _native.inject_device_alloc_failure(after)
        try:
            t = _run(m)
            assert np.array_equal(t, base)  # the failure point lies past this run's allocations
        except _native.EngineError as ex:
            failed += 1
            assert ex.code == -2 and "memory" in str(ex).lower(), str(ex)
        finally:
            _native.inject_device_alloc_failure(None)
    assert failed >= 10  # the run allocates at least that many buffers
    assert np.array_equal(_run(m), base)


def test_failed_growth_keeps_the_engine_as_it_was():
    m = W.closed_cube(n_per_species=2000)
    want = _run(m)
    h = W.model_handle(m, "fp32", seed=3)
    h.prepare()
    rng = np.random.default_rng(4)
    more = rng.uniform(-40, 40, size=(50_000, 3))  # needs a larger capacity
    _native.inject_device_alloc_failure(0)
    try:
        with pytest.raises(_native.EngineError) as ei:
            h.add_molecules(more, np.zeros(len(more), np.uint32))
        assert ei.value.code == -2
    finally:
        _native.inject_device_alloc_failure(None)
    assert int(h.counts().sum()) == 4000
    h.step(ITERS)
    assert np.array_equal(h.trajectory(ITERS), want)
    # the growth succeeds once memory is there
    h.add_molecules(more, np.zeros(len(more), np.uint32))
    assert int(h.counts().sum()) == int(want[-1].sum()) + len(more)
    h.close()


def test_server_fails_only_the_request_whose_admission_failed():
    ms = W.replica_models(3, seed=41, n_range=(1_000, 4_000), edge_range_um=(0.5, 1.0), levels=(2, 3))
    srv = _native.Server("fp32", 3, max_slots=4, autotune=False)
    try:
        h = W.model_handle(ms[0], "fp32", seed=700)
        t0 = srv.submit(h, 30)
        h.close()
        assert srv.wait(t0, 120) == "done"
        h = W.model_handle(ms[1], "fp32", seed=701)
        _native.inject_device_alloc_failure(0)  # the admission's first device allocation
        try:
            t1 = srv.submit(h, 30)
            assert srv.wait(t1, 120) == "failed"
        finally:
            _native.inject_device_alloc_failure(None)
            h.close()
        with pytest.raises(_native.EngineError) as ei:
            srv.result(t1)
        assert "memory" in str(ei.value).lower()
        # the server goes on: the next request runs and equals the model run alone
        h = W.model_handle(ms[2], "fp32", seed=702)
        t2 = srv.submit(h, 30)
        h.close()
        assert srv.wait(t2, 120) == "done"
        e = W.engine_for(ms[2], "fp32", seed=702)
        e.step(30)
        assert np.array_equal(srv.result(t2)[1], e.trajectory(30))
        e.close()
        assert srv.stats()["failed"] == 0  # the server itself never failed
    finally:
        srv.close()
