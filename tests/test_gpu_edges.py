"""Edge cases of the whole step: the subpartition grid, and ragged or empty replicas.

The subpartition grid only decides which walls and partners a move examines. On any
grid the reaction radius allows (R * sqrt(2) below half an edge), every wall a move
can hit and every partner within R of it is examined, collisions are ordered by time
and then partner id, and every draw is keyed by molecule id and iteration; so the
trajectories of a model cut into a coarse grid, into its own 0.1 um grid and into the
finest grid the radius allows (where occupants are binned per subpartition instead of
per octant, the key space being too large for octants) are the same, molecule for
molecule. Replicas of 0, 1, 31 and 33 molecules (empty, one lane, either side of a
warp) beside a larger one step exactly as they do alone. A model with the largest
species count (16) keeps its reaction bookkeeping.
"""
import numpy as np
import pytest

from mcell_gb300 import _native
from mcell_gb300 import workloads as W
from tests import harness as H

pytestmark = pytest.mark.gpu

NSP = 3


def _finest_grid(sc):
    # largest n with R * sqrt(2) < (edge / n) / 2
    n = int(np.floor(sc.partition_edge / (2.0 * 1.41421356238 * sc.rxn_radius)))
    while n > 1 and not sc.rxn_radius * 1.41421356238 < sc.partition_edge / n / 2.0:
        n -= 1
    return min(n, 300)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_trajectory_does_not_depend_on_the_subpartition_grid(precision):
    rng = np.random.default_rng(31)
    sc = H.sphere_in_cube_scene(rng, levels=2, n_mol=6000, p_rxn=0.3)
    grids = [sc.nsub, 7, _finest_grid(sc)]
    assert grids[2] > 2 * grids[0] and grids[2] ** 3 * NSP * 8 > (1 << 26)  # octants off on the finest
    iters = 20
    runs = []
    for n in grids:
        sc.nsub = n
        e = H.make_gpu_engine(sc, precision, bimol=[(0, 1, 0.3, (2, -1))], unimol=[(2, 0.05, (-1, -1))], seed=17)
        e.step(iters)
        tr = e.trajectory(iters)
        pos, sp, ids = e.molecules()
        o = np.argsort(ids)
        runs.append((tr, pos[o], sp[o], ids[o]))
        e.close()
    assert runs[0][0][-1, 2] > 0  # reactions happened
    for n, r in zip(grids[1:], runs[1:]):
        for a, b, what in zip(runs[0], r, ("counts", "positions", "species", "ids")):
            assert np.array_equal(a, b), f"{what} differ between {grids[0]} and {n} subpartitions per edge"


def _alone(model, precision, seed, iters):
    e = W.engine_for(model, precision, seed=seed)
    e.step(iters)
    t = e.trajectory(iters)
    pos, sp, ids = e.molecules()
    o = np.argsort(ids)
    e.close()
    return t, pos[o], sp[o]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ragged_and_empty_replicas_step_as_they_do_alone(precision):
    ms = W.replica_models(5, seed=41, n_range=(2_000, 6_000), edge_range_um=(0.5, 1.0), levels=(2, 3))
    for m, n in zip(ms, (0, 1, 31, 33)):
        m.pos, m.species = m.pos[:n], m.species[:n]
    iters = 25
    want = [_alone(m, precision, 500 + k, iters) for k, m in enumerate(ms)]
    b = _native.Batch(precision, NSP, len(ms))
    hs = [W.model_handle(m, precision, seed=500 + k) for k, m in enumerate(ms)]
    ids = b.add(hs)
    for h in hs:
        h.close()
    b.step(iters)
    for k, r in enumerate(ids):
        t = b.trajectory(r, iters)
        assert np.array_equal(t, want[k][0]), f"replica {k}"
        pos, sp, uid = b.molecules(r)
        o = np.argsort(uid)
        assert np.array_equal(pos[o], want[k][1]) and np.array_equal(sp[o], want[k][2]), f"replica {k}"
    assert int(b.counts(ids[0]).sum()) == 0
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sixteen_species(precision):
    """The largest species count (16), each species with its own diffusion step: seven
    pairs A_k + B_k -> P with products 14 and 15. Each reaction takes one of each
    reactant and makes one product, and no molecule leaves the box."""
    rng = np.random.default_rng(43)
    nsp = 16
    sc = H.cube_scene(rng, n_mol=30000, nsub=24)
    sc.mol_species = rng.integers(0, 14, size=30000).astype(np.uint32)
    sc.space_steps = np.linspace(1.0, 2.5, nsp)
    sc.wall_class = np.zeros((len(sc.tris), nsp), np.uint8)
    bimol = [(2 * k, 2 * k + 1, 0.2 + 0.05 * k, (14 + k % 2, -1)) for k in range(7)]
    init = np.bincount(sc.mol_species, minlength=nsp).astype(np.int64)
    e = H.make_gpu_engine(sc, precision, bimol=bimol, seed=4)
    e.step(30)
    c = e.counts().astype(np.int64)
    for k in range(7):
        assert c[2 * k] - c[2 * k + 1] == init[2 * k] - init[2 * k + 1], k
    assert (init[:14] - c[:14]).sum() == 2 * (c[14] + c[15])
    assert c[14] > 0 and c[15] > 0
    pos, sp, ids = e.molecules()
    assert len(ids) == int(c.sum()) and (np.abs(pos) <= 50 + 1e-3).all()
    assert np.array_equal(np.bincount(sp, minlength=nsp), c)
    e.close()


def test_counts_read_while_the_next_iteration_runs():
    """mcg_request_counts / mcg_wait_counts: the counts of every iteration, read one
    iteration late (the device runs the next meanwhile), equal the count trajectory;
    a request before the first iteration gives the uploaded counts; a slot taken by a
    later request makes the old ticket's wait fail."""
    rng = np.random.default_rng(8)
    sc = H.cube_scene(rng, n_mol=20000)
    e = H.make_gpu_engine(sc, "fp32", bimol=[(0, 1, 0.3, (2, -1))], seed=3)
    t0 = e.request_counts()
    assert np.array_equal(e.wait_counts(t0), e.counts())
    prev, seen = None, []
    for _ in range(6):
        e.step(1)
        t = e.request_counts()
        if prev is not None:
            seen.append(e.wait_counts(prev))
        prev = t
    seen.append(e.wait_counts(prev))
    assert np.array_equal(np.array(seen), e.trajectory(6))
    assert seen[-1][2] > 0
    e.step(2)
    tickets = [e.request_counts() for _ in range(8)]
    assert np.array_equal(e.wait_counts(tickets[0]), e.counts())
    e.request_counts()
    with pytest.raises(_native.EngineError):
        e.wait_counts(tickets[0])
    assert np.array_equal(e.wait_counts(tickets[1]), e.counts())
    e.close()
