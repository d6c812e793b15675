"""mcg_trace_cases_static (fixed device scratch, no device allocation) against
mcg_trace_cases (buffers allocated per call), both through the C ABI.

Both calls run the same trace kernel on the same inputs, so the tolerance is
zero: every result double must be identical, on two static calls in a row.
The file name sorts last so that the test also runs after every other test.
"""
import numpy as np
import pytest

from tests import harness as H
from mcell_gb300 import _native

pytestmark = pytest.mark.gpu

MAX_CASES = 256
MAX_DRAWS = 16384
MCG_ERR_ARG = -1


def _scene_and_cases(seed, n_cases):
    rng = np.random.default_rng(seed)
    sc = H.sphere_in_cube_scene(rng, levels=3, n_mol=4000, radius_um=0.6, cube_um=1.5, p_rxn=0.4)
    cases = H.random_cases(rng, sc, n_cases, scale=3.0, near_wall_frac=0.5)
    ids = np.array([c[0] for c in cases], np.uint64)
    disps = np.array([c[1] for c in cases])
    draws = np.array([c[2] for c in cases])
    return sc, ids, disps, draws


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_trace_matches_allocating_trace(precision):
    sc, ids, disps, draws = _scene_and_cases(11, MAX_CASES)
    e = H.engine_from_scene(sc, precision)
    want = e.trace_cases(ids, disps, draws)
    first = e.trace_cases_static(ids, disps, draws)
    second = e.trace_cases_static(ids, disps, draws)
    assert np.array_equal(first, want)
    assert np.array_equal(second, want)
    # a smaller request after a full one: results do not depend on what the scratch held
    part = e.trace_cases_static(ids[:17], disps[:17], draws[:17])
    assert np.array_equal(part, want[:17])
    e.close()


def test_static_trace_takes_no_device_memory():
    """The property the entry point exists for: with the next device allocation armed
    to fail, a static call still succeeds (it makes none), and the device's free
    memory is the same before and after the call."""
    torch = pytest.importorskip("torch")
    sc, ids, disps, draws = _scene_and_cases(13, 64)
    e = H.engine_from_scene(sc, "fp32")
    want = e.trace_cases_static(ids, disps, draws)
    free0 = torch.cuda.mem_get_info(0)[0]
    _native.inject_device_alloc_failure(0)
    try:
        got = e.trace_cases_static(ids, disps, draws)
        free1 = torch.cuda.mem_get_info(0)[0]
        # the armed failure is still pending (the static call made no allocation):
        # the allocating trace, which allocates, meets it
        with pytest.raises(_native.EngineError):
            e.trace_cases(ids, disps, draws)
    finally:
        _native.inject_device_alloc_failure(None)
    assert np.array_equal(got, want)
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes across the call"
    e.close()


def test_static_trace_rejects_oversized_and_unknown_requests():
    sc, ids, disps, draws = _scene_and_cases(12, 8)
    e = H.engine_from_scene(sc, "fp64")
    too_many = np.zeros(MAX_CASES + 1, np.uint64)
    with pytest.raises(_native.EngineError) as ex:
        e.trace_cases_static(too_many, np.zeros((MAX_CASES + 1, 3)), np.zeros((MAX_CASES + 1, 1), np.uint32))
    assert ex.value.code == MCG_ERR_ARG and "exceeds the maximum" in str(ex.value)
    per_case = MAX_DRAWS // 4 + 1
    with pytest.raises(_native.EngineError) as ex:
        e.trace_cases_static(ids[:4], disps[:4], np.zeros((4, per_case), np.uint32))
    assert ex.value.code == MCG_ERR_ARG and "draws_per_case" in str(ex.value)
    with pytest.raises(_native.EngineError) as ex:
        e.trace_cases_static(np.array([10 ** 12], np.uint64), disps[:1], draws[:1])
    assert ex.value.code == MCG_ERR_ARG and "not live" in str(ex.value)
    # the engine is still usable and agrees with the allocating trace afterwards
    assert np.array_equal(e.trace_cases_static(ids, disps, draws), e.trace_cases(ids, disps, draws))
    e.close()
