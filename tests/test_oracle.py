"""CPU tests: the oracle port against the reference's own routines.

1. against the golden fixtures (made from the reference routines by
   tests/golden/make_golden.py; these run everywhere),
2. against the reference routines directly on fresh random cases (only where
   oracle/_ref was built from the reference sources),
3. the oracle's serial engine against closed forms (diffusion, unimolecular
   decay, conservation), which also pins the rate -> probability conversion.
"""
import numpy as np
import pytest

from tests import harness as H
from mcell_gb300 import conversion


@pytest.mark.parametrize("name", H.GOLDEN_SCENES)
def test_oracle_matches_golden(name):
    sc, g = H.load_golden(name)
    orc = H.oracle().scene(sc)
    assert np.array_equal(orc.info(), g["info"])
    assert np.array_equal(orc.wall_consts(len(sc.tris)), g["wall_consts"]), "wall constants differ"
    counts, lst = orc.walls_in_subparts(sc.nsub ** 3)
    assert np.array_equal(counts, g["wsp_counts"]) and np.array_equal(lst, g["wsp_list"]), "wall binning differs"
    got = np.array([orc.diffuse_case(int(m), d, dr) for m, d, dr in zip(g["mols"], g["disps"], g["draws"])])
    bad = H.compare_results(got, g["results"], rel=0.0, scene=sc)
    # exact_disk with 2+ occluding edges uses an angular sweep here, so allow 1e-9 there
    bad = [c for c in bad if H.compare_results(got[c:c + 1], g["results"][c:c + 1], rel=1e-9, scene=sc)]
    assert not bad, f"{len(bad)} cases differ, first {bad[:5]}"


def test_reaction_tests_match_golden():
    z = np.load(H.GOLDEN / "rxn_tests.npz")
    orc = H.oracle()
    tb = np.array([orc.test_bimolecular(p, s, u) for p, s, u in zip(z["P"], z["S"], z["U"])])
    # the reference returns the pathway (0) or PATHWAY_INDEX_NO_RXN (< 0)
    assert np.array_equal(tb >= 0, z["bimol"] >= 0)
    tu = np.array([orc.time_of_unimol(k, u) for k, u in zip(z["K"], z["Uu"])])
    assert np.array_equal(tu, z["unimol"])


def test_reaction_pathways_match_golden():
    """Classes of 1-4 pathways: test_bimolecular's fire decision and pathway, and
    which_unimolecular's pathway, against the reference's routines (golden)."""
    z = np.load(H.GOLDEN / "rxn_pathways.npz")
    orc = H.oracle()
    tb = np.array([orc.test_bimolecular_pw(z["cum"][i, :z["npw"][i]], z["scaling"][i], z["U"][i])
                   for i in range(len(z["U"]))])
    assert np.array_equal(np.where(tb < 0, -1, tb), np.where(z["bimol"] < 0, -1, z["bimol"]))
    tu = np.array([orc.which_unimolecular(z["ucum"][i, :z["unpw"][i]], z["Uu"][i]) for i in range(len(z["Uu"]))])
    assert np.array_equal(tu, z["unimol"])
    assert len(np.unique(z["bimol"])) >= 4 and len(np.unique(z["unimol"])) == 4


REF = H.reference(64)


@pytest.mark.skipif(REF is None, reason="reference routines not built here (no reference sources)")
def test_oracle_pathways_match_reference_random():
    rng = np.random.default_rng(13)
    for _ in range(2000):
        k = int(rng.integers(1, 5))
        cum = np.cumsum(rng.uniform(0, 0.7, k)) * (3.0 if rng.random() < 0.2 else 1.0)
        sc, u = float(rng.uniform(0, 2)), int(rng.integers(0, 2 ** 32))
        a, b = H.oracle().test_bimolecular_pw(cum, sc, u), REF.test_bimolecular_pw(cum, sc, u)
        assert (a < 0 and b < 0) or a == b
        assert H.oracle().which_unimolecular(cum, u) == REF.which_unimolecular(cum, u)


@pytest.mark.skipif(REF is None, reason="reference routines not built here (no reference sources)")
@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_matches_reference_random(seed):
    rng = np.random.default_rng(seed)
    star = H.star_scene(rng, n_mol=2000)
    star.rxn_p = np.array([0.3])
    for sc in [H.cube_scene(rng, n_mol=1500, p_rxn=0.3),
               H.sphere_in_cube_scene(rng, levels=3, n_mol=2000, radius_um=0.6, cube_um=1.5, p_rxn=0.3), star]:
        o, r = H.oracle().scene(sc), REF.scene(sc)
        assert np.array_equal(o.wall_consts(len(sc.tris)), r.wall_consts(len(sc.tris)))
        n3 = sc.nsub ** 3
        co, lo = o.walls_in_subparts(n3)
        cr, lr = r.walls_in_subparts(n3)
        assert np.array_equal(co, cr) and np.array_equal(lo, lr)
        bad = 0
        for m, d, dr in H.random_cases(rng, sc, 800, scale=3.0, near_wall_frac=0.5):
            a, b = o.diffuse_case(m, d, dr), r.diffuse_case(m, d, dr)
            if not np.array_equal(a, b) and H.compare_results(a[None], b[None], rel=1e-9, scene=sc):
                bad += 1
        assert bad == 0


# ---------------------------------------------------------------- serial engine closed forms

def test_oracle_engine_conserves_and_confines():
    rng = np.random.default_rng(3)
    sc = H.cube_scene(rng, n_mol=500)
    e = H.make_oracle_engine(sc)
    counts = e.run(50)
    assert (counts.sum(1) == 500).all()
    pos, _ = e.molecules()
    assert (np.abs(pos) <= 50).all()


def test_oracle_engine_unimolecular_decay():
    rng = np.random.default_rng(4)
    sc = H.cube_scene(rng, n_mol=4000)
    sc.mol_species[:] = 2
    k = 1e-2
    e = H.make_oracle_engine(sc, unimol=[(2, k, (-1, -1))])
    counts = e.run(100)
    n = counts[:, 2].astype(float)
    t = np.arange(1, 101)
    expect = 4000 * np.exp(-k * t)
    assert np.all(np.abs(n - expect) < 5 * np.sqrt(expect * (1 - np.exp(-k * t))) + 1)


def test_space_step_and_probability_conversions():
    lu = conversion.length_unit_um()
    assert lu == 0.01
    assert abs(conversion.space_step(1e-6, 1e-6, lu) - 2.0) < 1e-12
    R = conversion.default_rxn_radius_um()
    p = conversion.bimol_probability(1e8, 2.0, 2.0, R, 1e-6, lu)
    assert abs(p - 0.0368) < 5e-4
    lay = conversion.partition_layout([-0.5] * 3, [0.5] * 3, partition_dimension_um=1.2,
                                      subpartition_dimension_um=0.1)
    assert lay.nsub == 12 and abs(lay.edge - 120) < 1e-9 and abs(lay.origin[0] + 60) < 1e-9


@pytest.mark.parametrize("name,iters", [("closed_cube", 100), ("sphere_in_cube", 40)])
def test_ensemble_fixture_reproduces_from_the_oracle(name, iters):
    """The committed ensemble fixture (tests/golden/make_ensembles.py) is what the
    oracle's serial engine computes now: seed 1, the first rows."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_ensembles", H.GOLDEN / "make_ensembles.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    z = np.load(H.GOLDEN / f"ensemble_{name}.npz")
    assert int(z["seeds"][0]) == 1
    got = mk.run_one((name, 1, iters))
    assert np.array_equal(got, z["counts"][0, :iters // int(z["every"])])


def _exact_disk_cases(rng, sc, pos, n_cases):
    sc.mol_pos = pos
    o, r = H.oracle().scene(sc), REF.scene(sc)
    R, n = sc.rxn_radius, len(pos)
    got, want = [], []
    for _ in range(n_cases):
        t, m = int(rng.integers(0, n)), int(rng.integers(0, n))
        if m == t:
            continue
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        off = rng.normal(size=3)
        off -= off.dot(d) * d
        off *= rng.uniform(0, R) / np.linalg.norm(off)
        loc, mv = pos[t] + off, d * rng.uniform(0.5, 3.0)
        got.append(o.exact_disk(loc, mv, m, t))
        want.append(r.exact_disk(loc, mv, m, t))
    return np.array(got), np.array(want)


@pytest.mark.skipif(REF is None, reason="reference routines not built here (no reference sources)")
def test_exact_disk_against_the_reference_next_to_edges_and_vertices():
    """exact_disk at collision points within R of several walls: next to the closed
    cube's edges and corners, and next to the vertices of the star, where many small
    triangles meet (2+ occluding edges). 0 or 1 edge is the reference's arithmetic; 2+
    edges are an angular sweep of the exact visible area, while the reference merges
    vertices and radii closer than POS_EPS (exact_disk_utils.inl:652-733): measured,
    all of 20,000 cube cases within 1e-9 and 3 of 120,000 star cases beyond it (at
    most 5e-8)."""
    rng = np.random.default_rng(1)
    sc = H.cube_scene(rng, n_mol=400)
    R, half = sc.rxn_radius, 50.0
    pos = np.zeros((400, 3))
    for i in range(400):
        c = rng.choice([-1, 1], size=3) * half
        p = rng.uniform(-half + 2, half - 2, size=3)
        for a in rng.choice(3, size=int(rng.integers(1, 4)), replace=False):
            p[a] = c[a] - np.sign(c[a]) * rng.uniform(0.0, 1.5 * R)
        pos[i] = p
    st = H.star_scene(rng, n_mol=400)
    v = st.verts[np.unique(st.tris[st.obj == 0])]
    spos = v[rng.integers(0, len(v), 400)] + rng.normal(size=(400, 3)) * 0.5 * st.rxn_radius
    for scene, p in ((sc, pos), (st, spos)):
        got, want = _exact_disk_cases(rng, scene, p, 10000)
        assert np.array_equal(got < 0, want < 0)
        rel = np.abs(got - want) / np.maximum(1.0, np.abs(want))
        assert (got == want).mean() > 0.8
        assert (rel <= 1e-9).mean() > 0.999 and rel.max() <= 1e-7
        assert ((want > 0) & (want < 1)).sum() > 2000  # occluded disks, not only free ones
