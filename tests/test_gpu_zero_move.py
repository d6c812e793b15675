"""A transparent wall met exactly at the end of a move (t = 1) leaves a zero move.

The trace loops while a wall was hit (diffuse_react_event.cpp:450-618), so the zero
move is traced again. Its partner test, collide_mol (collision_utils.inl:464-515),
divides by the squared move length: without a guard every occupant of the scanned
octants passes its tests with t = 0 / 0 (NaN), and a reaction at a NaN time and place
follows. The engine scans no partners for a zero move. In fp32 a crossing time rounds
to 1 far more often than in fp64; a 1,000-iteration run of the batching workload met it.
"""
import numpy as np
import pytest

from mcell_gb300 import geometry
from tests import harness as H

pytestmark = pytest.mark.gpu


def _scene():
    v, w = geometry.create_box(edge_dimension=1.0)
    verts = v / 0.01  # internal units: the box spans [-50, 50]
    # a transparent square (for A) in the plane x = 3
    sq = np.array([[3.0, -40.0, -40.0], [3.0, 40.0, -40.0], [3.0, 40.0, 40.0], [3.0, -40.0, 40.0]])
    verts = np.vstack([verts, sq])
    n0 = len(v)
    tris = np.vstack([w, [[n0, n0 + 1, n0 + 2], [n0, n0 + 2, n0 + 3]]]).astype(np.uint32)
    wc = np.zeros((len(tris), 3), np.uint8)
    wc[-2:, 0] = 1
    pos = [[-2.0, 0.3, 0.2]]
    # B molecules in the subpartition where the move ends (two in the octant of the end
    # point, which the partner scan reads), none near the segment
    pos += [[4.5, 3.0, 3.0], [1.0, 4.0, 2.0], [5.0, 5.0, 5.0], [7.0, 2.0, 8.0], [4.0, 6.5, 1.5]]
    sp = np.array([0] + [1] * 5, np.uint32)
    return H.Scene(np.array([-60.0, -60.0, -60.0]), 120.0, 12, 0.5, verts, tris,
                   np.array([2.0, 2.0, 1.414213562373095]), wc, np.array([[0, 1]], np.uint32),
                   np.array([1.0]), np.array(pos), sp)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_crossing_at_the_end_of_the_move_meets_no_partner(precision):
    sc = _scene()
    e = H.engine_from_scene(sc, precision)
    disp = np.array([[5.0, 0.0, 0.0]])  # from x = -2 to the plane x = 3: t = 1 exactly
    draws = np.full((1, 64), 12345, np.uint32)
    got = e.trace_cases(np.array([0], np.uint64), disp, draws)[0]
    assert np.isfinite(got).all()
    assert got[0] == 0  # finished: no reaction, no error
    n_ev = int(got[6])
    ev = got[9:9 + 8 * n_ev].reshape(-1, 8)
    assert n_ev == 1 and ev[0, 0] == 2  # one event: the transparent crossing
    # the crossing point; the zero move lies in the plane of the square's other triangle,
    # whose re-try (jump_away_line) may move it by the fp64 jump
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.allclose(got[1:4], [3.0, 0.3, 0.2], rtol=0, atol=tol)
    e.close()
