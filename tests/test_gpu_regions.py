"""Releases into region expressions, by concentration, and vacuums, on the device,
pinned to the reference's ReleaseEvent::release_inside_regions (release_event.cpp:904-
952; is_point_inside_region_expr_recursively :785-810, num_vol_mols_from_conc
:826-856, vacuum_inside_regions :864-896, randomly_remove_molecules :578-597) on the
three-object scene of tests/harness.regions_scene (golden fixture
tests/golden/regions.npz):

- the parity harness (mcg_release_region_harness) draws from the fixture's injected
  streams in one device thread: released positions, counts and draws taken bit for
  bit (the inside tests run in fp64 in both engines), and the molecules a vacuum
  removes (chosen on the host from the device's candidates in id order);
- the production call (mcg_release_region): placed molecules lie inside their
  expression, the exact concentration count is the reference's, a vacuum removes the
  chosen number of the species' molecules inside and no other.
"""
import numpy as np
import pytest

from mcell_gb300 import _native
from tests import harness as H

pytestmark = pytest.mark.gpu

G = np.load(H.GOLDEN / "regions.npz")


def _engine(precision, seed=1):
    e = _native.Engine(precision, G["origin"], float(G["partition_edge"]), int(G["nsub"]), float(G["rxn_radius"]), 3,
                       seed=seed)
    e.set_species([2.0, 2.0, 1.414213562373095])
    e.upload_mesh(G["verts"], G["tris"], np.zeros((len(G["tris"]), 3), np.uint8))
    e.set_wall_objects(G["obj"])
    e.add_molecules(G["mol_pos"], G["mol_species"])
    e.prepare()
    return e


def _expr(k):
    return G["expr"][k, :G["n_expr"][k]].tolist()


def _inside_expr(e, tokens, pos):
    """The expression evaluated from the engine's own per-object inside tests."""
    st = []
    for t in tokens:
        if t >= 0:
            st.append(e.inside_tests(pos, "object", t) == 1)
        else:
            b, a = st.pop(), st.pop()
            st.append(a | b if t == -1 else (a & b if t == -2 else a & ~b))
    return st[0]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_harness_matches_the_reference(precision):
    e = _engine(precision)
    for c, (k, method, number) in enumerate(G["cases"]):
        conc = float(G["case_conc"][c]) if method == 1 else None
        pos, removed, used = e.release_region_harness(0, _expr(k), G["draws"][c], number=int(number),
                                                      concentration=conc)
        assert used == G["used"][c], (c, used, G["used"][c])
        if number < 0:
            assert np.array_equal(removed.astype(np.int64), G["removed"][c, :G["n_removed"][c]]), c
            assert len(pos) == 0
        else:
            want = G["pos"][c, :G["n_pos"][c]]
            assert len(pos) == len(want), (c, len(pos), len(want))
            assert np.array_equal(pos, want), c
    e.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_release_into_an_expression(precision):
    e = _engine(precision)
    n0 = len(G["mol_species"])
    tokens = [1, 0, -3]  # in the box, not in the star
    assert e.release_region(1, tokens, number=500, seed=3) == 500
    pos, sp, ids = e.molecules()
    new = ids >= n0
    assert new.sum() == 500 and (sp[new] == 1).all()
    assert sorted(ids[new].tolist()) == list(range(n0, n0 + 500))
    inside = _inside_expr(e, tokens, pos[new])
    # fp32 stores the points rounded: one within an ulp of a wall may test outside
    assert inside.all() if precision == "fp64" else inside.sum() >= 498
    # one object by concentration: the reference's exact count
    c = next(i for i, (k, m, n) in enumerate(G["cases"]) if m == 1 and G["n_expr"][k] == 1)
    k = int(G["cases"][c][0])
    done = e.release_region(0, _expr(k), concentration=float(G["case_conc"][c]), seed=4)
    assert done == G["computed"][c]
    # an expression by concentration: that many draws, each placing one molecule if inside
    c = next(i for i, (k, m, n) in enumerate(G["cases"]) if m == 1 and G["n_expr"][k] > 1)
    k = int(G["cases"][c][0])
    lo, hi = G["bbox"][k, :3], G["bbox"][k, 3:]
    n_draws = int(6.0221417930e23 * 1e-15 * G["case_conc"][c] * np.prod(hi - lo) * 0.01 ** 3 + 0.5)
    before = len(e.molecules()[2])
    done = e.release_region(0, _expr(k), concentration=float(G["case_conc"][c]), seed=5)
    assert 0 < done <= n_draws and len(e.molecules()[2]) == before + done
    # molecules added afterwards get ids of their own
    e.add_molecules(G["mol_pos"][:10], G["mol_species"][:10])
    ids = e.molecules()[2]
    assert len(np.unique(ids)) == len(ids)
    e.step(3)
    e.sync()
    e.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_vacuum_removes_inside_only(precision):
    e = _engine(precision)
    tokens = [2, 0, -3]  # the small cube outside the star
    pos, sp, ids = e.molecules()
    inside = _inside_expr(e, tokens, pos) & (sp == 0)
    m = int(inside.sum())
    assert m > 10
    removed = -e.release_region(0, tokens, number=-(m // 2), seed=9)
    assert removed == m // 2
    pos2, sp2, ids2 = e.molecules()
    gone = set(ids.tolist()) - set(ids2.tolist())
    assert len(gone) == removed and len(ids2) == len(ids) - removed
    assert all(inside[ids.tolist().index(g)] for g in gone)
    # more than there are: all of them
    assert -e.release_region(0, tokens, number=-10 * m, seed=10) == m - removed
    pos3, sp3, _ = e.molecules()
    assert not (_inside_expr(e, tokens, pos3) & (sp3 == 0)).any()
    e.close()


def test_invalid_region_release_is_refused():
    e = _engine("fp32")
    for bad in ([0, -1], [5], [0, 1, 2, -1]):
        with pytest.raises(_native.EngineError):
            e.release_region(0, bad, number=10)
    with pytest.raises(_native.EngineError):
        e.release_region(7, [0], number=10)  # no such species
    e.close()


def _handle(precision, seed):
    h = _native.Engine(precision, G["origin"], float(G["partition_edge"]), int(G["nsub"]), float(G["rxn_radius"]), 3,
                       seed=seed)
    h.set_species([2.0, 2.0, 1.414213562373095])
    h.upload_mesh(G["verts"], G["tris"], np.zeros((len(G["tris"]), 3), np.uint8))
    h.set_wall_objects(G["obj"])
    h.add_molecules(G["mol_pos"], G["mol_species"])
    return h


def test_batch_release_into_one_replica():
    b = _native.Batch("fp32", 3, 2)
    hs = [_handle("fp32", 1), _handle("fp32", 2)]
    ids = b.add(hs)
    for h in hs:
        h.close()
    def species_counts(r):
        return np.bincount(b.molecules(r)[1], minlength=3)

    c0, c1 = species_counts(ids[0]), species_counts(ids[1])
    assert b.release_region(ids[1], 2, [1, 0, -3], number=300, seed=5) == 300
    removed = -b.release_region(ids[0], 0, [2, 0, -3], number=-5, seed=6)
    assert removed == 5
    assert (species_counts(ids[1]) - c1).tolist() == [0, 0, 300]
    assert (c0 - species_counts(ids[0])).tolist() == [5, 0, 0]
    b.step(2)
    b.sync()
    b.close()
