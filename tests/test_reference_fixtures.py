"""The golden fixtures of the diffusion cases, the reaction decisions, the inside tests
and the region releases reproduce from the reference's own routines (oracle/_ref, compiled from the reference sources by
oracle/ref/build_ref.py where those sources exist; skipped elsewhere): the recorded
decisions, volumes, boxes, counts, positions and removals are what the reference
computes now, on the recorded inputs."""
import numpy as np
import pytest

from tests import harness as H

REF = H.reference(64)
pytestmark = pytest.mark.skipif(REF is None, reason="oracle/_ref not built (reference sources absent)")


def test_region_fixture_reproduces():
    z = np.load(H.GOLDEN / "regions.npz")
    sc = H.regions_scene(np.random.default_rng(0))
    sc.origin, sc.partition_edge, sc.nsub = z["origin"], float(z["partition_edge"]), int(z["nsub"])
    sc.verts, sc.tris, sc.obj = z["verts"], z["tris"], z["obj"]
    sc.mol_pos, sc.mol_species = z["mol_pos"], z["mol_species"]
    h = REF.scene(sc)
    h.set_objects(sc.obj, [0, 0, 0])
    assert np.array_equal([h.region_volume(o) for o in range(3)], z["volumes"])
    for k in range(len(z["n_expr"])):
        e = z["expr"][k, :z["n_expr"][k]].tolist()
        assert np.array_equal(np.concatenate(h.region_expr_bbox(e)), z["bbox"][k])
    for d, c, n in zip(z["conc_dia"], z["conc"], z["conc_n"]):
        assert REF.number_from_concentration(d, c, 0.01) == n
    for c, (k, method, number) in enumerate(z["cases"]):
        e = z["expr"][k, :z["n_expr"][k]].tolist()
        computed, pos, rem, used = h.release_inside_regions(
            e, z["draws"][c], number=int(number), species=0,
            concentration=float(z["case_conc"][c]) if method == 1 else None)
        assert computed == z["computed"][c] and used == z["used"][c]
        assert np.array_equal(pos, z["pos"][c, :z["n_pos"][c]])
        assert np.array_equal(rem.astype(np.int64), z["removed"][c, :z["n_removed"][c]])


def test_inside_fixture_reproduces():
    z = np.load(H.GOLDEN / "inside_star.npz")
    sc = H.star_scene(np.random.default_rng(0))
    sc.origin, sc.partition_edge, sc.nsub = z["origin"], float(z["partition_edge"]), int(z["nsub"])
    sc.verts, sc.tris, sc.obj = z["verts"], z["tris"], z["obj"]
    h = REF.scene(sc)
    h.set_objects(sc.obj, [1, 1])
    pts = z["points"][::7]
    cv = np.array([h.counted_volume_for_pos(p) for p in pts], np.uint32)
    reg = np.array([[h.inside_region(o, p) for o in (0, 1)] for p in pts], np.int32)
    assert np.array_equal(cv, z["counted"][::7])
    assert np.array_equal(reg, z["inside_region"][::7])
    for k in range(len(z["rel_shape"])):
        n = int(z["rel_n"][k])
        pos, used = REF.release_ellipsoid_or_rectcuboid(int(z["rel_shape"][k]), n, z["rel_loc"][k], z["rel_dia"][k],
                                                        z["rel_draws"][k])
        assert used == int(z["rel_used"][k]) and np.array_equal(pos, z["rel_pos"][k, :n]), k


@pytest.mark.parametrize("name", H.GOLDEN_SCENES)
def test_diffusion_fixture_reproduces(name):
    """Every recorded diffusion case, its wall constants and wall lists, from the
    reference routines now, bit for bit."""
    sc, g = H.load_golden(name)
    r = REF.scene(sc)
    assert np.array_equal(r.wall_consts(len(sc.tris)), g["wall_consts"])
    counts, lst = r.walls_in_subparts(sc.nsub ** 3)
    assert np.array_equal(counts, g["wsp_counts"]) and np.array_equal(lst, g["wsp_list"])
    got = np.array([r.diffuse_case(int(m), d, dr) for m, d, dr in zip(g["mols"], g["disps"], g["draws"])])
    assert not H.compare_results(got, g["results"], rel=0.0, scene=sc)


def test_reaction_fixtures_reproduce():
    """test_bimolecular, time_of_unimol and which_unimolecular on the recorded draws."""
    z = np.load(H.GOLDEN / "rxn_tests.npz")
    tb = np.array([REF.test_bimolecular(p, s, u) for p, s, u in zip(z["P"], z["S"], z["U"])])
    assert np.array_equal(tb, z["bimol"])
    tu = np.array([REF.time_of_unimol(k, u) for k, u in zip(z["K"], z["Uu"])])
    assert np.array_equal(tu, z["unimol"])
    w = np.load(H.GOLDEN / "rxn_pathways.npz")
    tb = np.array([REF.test_bimolecular_pw(w["cum"][i, :w["npw"][i]], w["scaling"][i], w["U"][i])
                   for i in range(len(w["U"]))])
    assert np.array_equal(tb, w["bimol"])
    tu = np.array([REF.which_unimolecular(w["ucum"][i, :w["unpw"][i]], w["Uu"][i]) for i in range(len(w["Uu"]))])
    assert np.array_equal(tu, w["unimol"])
