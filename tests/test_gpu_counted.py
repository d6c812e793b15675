"""Counted volumes: molecules inside a closed object, kept per molecule and set
at crossings, must equal a recount of the downloaded positions (the icosphere is
convex: inside = behind every face plane) — exactly in fp64."""
import numpy as np
import pytest

from mcell_gb300 import conversion, geometry
from mcell_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _model(n=40_000):
    lu = conversion.length_unit_um()
    sv, sw = geometry.create_icosphere(0.5, 3)
    bv, bw = geometry.create_box(edge_dimension=1.4)
    v, w, obj = geometry.merge_meshes((sv, sw), (bv, bw))
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=1.6, subpartition_dimension_um=0.1)
    steps, bimol, unimol = W._chemistry(1e-6, lu, conversion.default_rxn_radius_um(), k_unimol=1e3)
    rng = np.random.default_rng(5)
    pos = rng.uniform(-0.7 / lu, 0.7 / lu, size=(n, 3))
    sp = (np.arange(n) % 2).astype(np.uint32)
    wc = np.zeros((len(w), 3), np.uint8)
    wc[obj == 0, 0] = 1  # A crosses the sphere
    m = W.Model("counted", lay.origin, lay.edge, lay.nsub, conversion.default_rxn_radius_um() / lu, v / lu, w, wc,
                steps, bimol, unimol, pos, sp, 1e-6)
    return m, obj, sv / lu, sw


def _recount(pos, sp, sv, sw, nsp=3):
    a, b, c = sv[sw[:, 0]], sv[sw[:, 1]], sv[sw[:, 2]]
    n = np.cross(b - a, c - a)
    d = (n * a).sum(1)
    inside = ((pos @ n.T) - d < 0).all(1)
    return np.array([inside[sp == s].sum() for s in range(nsp)])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_counted_volume_follows_crossings(precision):
    m, obj, sv, sw = _model()
    h = W.model_handle(m, precision, seed=4)
    h.set_wall_objects(obj)
    h.set_counted_objects([0])
    h.prepare()
    pos, sp, _ = h.molecules()
    assert np.array_equal(h.counted_counts()[:, 0], _recount(pos, sp, sv, sw))
    h.step(30)
    traj = h.counted_trajectory(30)
    now = h.counted_counts()
    assert np.array_equal(traj[-1], now)
    pos, sp, _ = h.molecules()
    want = _recount(pos, sp, sv, sw)
    got = now[:, 0].astype(np.int64)
    if precision == "fp64":
        assert np.array_equal(got, want)
    else:
        assert np.abs(got - want).max() <= max(2, int(1e-4 * len(sp)))
    assert traj[:, 0, 0].std() > 0  # A moves in and out
    # a release inside the object: every new molecule counted inside
    before = h.counted_counts()[1, 0]
    h.release(1, 5000, "inside", obj=0, seed=3)
    assert h.counted_counts()[1, 0] == before + 5000
    h.close()
