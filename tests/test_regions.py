"""Host logic of releases into region expressions, by concentration, and of vacuums,
against the reference's own routines (tests/golden/regions.npz, recorded by
tests/golden/make_golden.py from oracle/_ref: Region::initialize_volume_info_if_needed,
compute_region_expr_bounding_box, calculate_number_to_release,
ReleaseEvent::randomly_remove_molecules). No GPU: these run in the C-ABI library's host
code (mcg_object_volume, mcg_region_expr_bbox, mcg_release_number_from_concentration,
mcg_vacuum_select). Bit-exact: the arithmetic is the reference's, in its order."""
import numpy as np
import pytest

from mcell_gb300 import _native
from tests import harness as H

G = np.load(H.GOLDEN / "regions.npz")


def _expr(k):
    return G["expr"][k, :G["n_expr"][k]].tolist()


def test_object_volumes_match_the_reference():
    for o in range(3):
        v = _native.object_volume(G["verts"], G["tris"], G["obj"].astype(np.uint16), o)
        assert v == G["volumes"][o], (o, v, G["volumes"][o])


def test_expression_boxes_match_the_reference():
    for k in range(len(G["n_expr"])):
        lo, hi = _native.region_expr_bbox(G["verts"], G["tris"], G["obj"].astype(np.uint16), _expr(k))
        assert np.array_equal(np.concatenate([lo, hi]), G["bbox"][k]), (k, lo, hi, G["bbox"][k])


def test_concentration_counts_match_the_reference():
    for d, c, n in zip(G["conc_dia"], G["conc"], G["conc_n"]):
        assert _native.release_number_from_concentration(d, c, 0.01) == n


def test_vacuum_choice_matches_the_reference():
    seen = 0
    for c, (k, method, number) in enumerate(G["cases"]):
        if number >= 0:
            continue
        m = int(G["n_candidates"][c])
        cand = G["candidates"][c, :m]
        chosen, used = _native.vacuum_select(m, int(-number), G["draws"][c])
        assert used == G["used"][c]
        want = G["removed"][c, :G["n_removed"][c]]
        assert np.array_equal(cand[chosen.astype(bool)], want), c
        seen += 1
    assert seen == 4


def test_invalid_region_expressions_are_refused():
    v, w, o = G["verts"], G["tris"], G["obj"].astype(np.uint16)
    for bad in ([], [0, -1], [0, 1], [3], [0, 1, -4], list(range(3)) * 5 + [-1]):
        with pytest.raises((_native.EngineError, KeyError, ValueError)):
            _native.region_expr_bbox(v, w, o, bad)
    with pytest.raises(_native.EngineError):
        _native.release_number_from_concentration([10, 10, 10], -1.0, 0.01)


def test_region_entry_points_check_their_arguments():
    import ctypes
    L = _native.lib()
    n = ctypes.c_uint32()
    assert L.mcg_vacuum_select(ctypes.c_uint32(3), ctypes.c_uint32(1), None, ctypes.c_uint32(0), None,
                               ctypes.byref(n)) == -1
    done = ctypes.c_int64()
    ex = np.array([0], np.int32)
    assert L.mcg_release_region(None, 0, 0, ctypes.c_int64(5), ctypes.c_double(0), ctypes.c_double(0.01),
                                ex.ctypes.data_as(ctypes.c_void_p), 1, ctypes.c_uint64(1), ctypes.byref(done)) == -1
    assert L.mcg_batch_release_region(None, 0, 0, 0, ctypes.c_int64(5), ctypes.c_double(0), ctypes.c_double(0.01),
                                      ex.ctypes.data_as(ctypes.c_void_p), 1, ctypes.c_uint64(1),
                                      ctypes.byref(done)) == -1
    vol = ctypes.c_double()
    assert L.mcg_object_volume(0, None, 0, None, None, 0, ctypes.byref(vol)) == -1
