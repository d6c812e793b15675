#!/usr/bin/env python3
"""Generates the golden fixtures in tests/golden/ from the reference's own routines.

Needs oracle/_ref/libmcell_ref{64,32}.so, which oracle/ref/build_ref.py compiles
from the reference sources (only possible where the reference tree exists).
Every case feeds an injected displacement and injected 32-bit draws to the
reference's ray_trace_vol / collide_wall / reflect_from_wall / exact_disk /
test_bimolecular path (driven as diffuse_vol_molecule does) and records the
result: status, final position and subpartition, draws used, and the event list
(wall reflections / crossings / absorptions, partners tested / reacted /
occluded, with times and positions).

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from tests import harness as H  # noqa: E402

NDRAWS = 24


def scenes(rng):
    out = {}
    sc = H.cube_scene(rng, n_mol=800, nsub=12, partition_um=1.2, p_rxn=0.0368)
    out["cube"] = sc
    sc = H.cube_scene(rng, n_mol=3000, nsub=12, partition_um=1.2, p_rxn=0.6)
    out["cube_dense"] = sc
    sc = H.cube_scene(rng, n_mol=600, nsub=12, partition_um=1.2, p_rxn=0.2)
    wc = np.zeros((12, 3), np.uint8)
    wc[[2, 8], 0] = 1     # x = +50 face transparent to A
    wc[[5, 11], 1] = 2    # z = +50 face absorptive for B
    wc[[0, 6], 0] = 2     # x = -50 face absorptive for A
    sc.wall_class = wc
    out["cube_classes"] = sc
    sc = H.sphere_in_cube_scene(rng, levels=2, n_mol=2500, radius_um=0.5, cube_um=1.2, p_rxn=0.5)
    out["sphere"] = sc
    return out


def add_edge_molecules(sc: H.Scene):
    cases = H.edge_cases(sc)
    extra = [
        ((50.0, 0.0, 0.0), (0.0, 3.0, 1.0)),    # on the wall plane, moving along it: REDO
        ((50.0, 3.0, 3.0), (-2.0, 0.5, 0.0)),   # on the wall plane, moving away
    ]
    cases = cases + extra
    n0 = len(sc.mol_species)
    pos = np.array([c[0] for c in cases])
    sc.mol_pos = np.concatenate([sc.mol_pos, pos])
    sc.mol_species = np.concatenate([sc.mol_species, np.zeros(len(cases), np.uint32)])
    return [(n0 + k, np.array(c[1])) for k, c in enumerate(cases)]


def partner_cases(rng, sc: H.Scene, n):
    """Displacements aimed past a reacting partner: the nearest molecule of a reacting
    species, passed within 1.2 R, overshooting by 5-60% (exercises collide_mol,
    exact_disk near walls and test_bimolecular)."""
    cases = []
    nm = len(sc.mol_species)
    react = {}
    for a, b in np.asarray(sc.rxn_ab).reshape(-1, 2):
        react.setdefault(int(a), set()).add(int(b))
        react.setdefault(int(b), set()).add(int(a))
    for _ in range(n):
        i = int(rng.integers(0, nm))
        ok = np.isin(sc.mol_species, list(react.get(int(sc.mol_species[i]), [])))
        ok[i] = False
        if not ok.any():
            continue
        d = sc.mol_pos - sc.mol_pos[i]
        dist = np.where(ok, np.linalg.norm(d, axis=1), np.inf)
        j = int(np.argmin(dist))
        v = d[j]
        L = np.linalg.norm(v)
        u = v / L
        w = np.cross(u, rng.normal(size=3))
        w /= np.linalg.norm(w)
        aim = v + w * rng.uniform(0, 1.2 * sc.rxn_radius)
        cases.append((i, aim * rng.uniform(1.05, 1.6)))
    return cases


def record_scene(ref64, rng, name, sc, cases):
    """Runs the cases through the reference's routines and writes diffuse_<name>.npz."""
    h = ref64.scene(sc)
    mols = np.array([c[0] for c in cases], np.uint32)
    disps = np.array([c[1] for c in cases], np.float64)
    draws = rng.integers(0, 2 ** 32, size=(len(cases), NDRAWS), dtype=np.uint64).astype(np.uint32)
    # a share of cases with draws that make reactions fire (small uniforms)
    draws[::3, :] = (draws[::3, :] >> 6).astype(np.uint32)
    res = np.array([h.diffuse_case(int(m), d, dr) for m, d, dr in zip(mols, disps, draws)])
    nev = int(res[:, 6].max())
    keep = H.RES_HDR + H.EV_SIZE * max(1, min(nev, H.EV_MAX))
    info = h.info()
    wc_ref = h.wall_consts(len(sc.tris))
    counts, lst = h.walls_in_subparts(sc.nsub ** 3)
    np.savez_compressed(
        HERE / f"diffuse_{name}.npz",
        origin=sc.origin, partition_edge=sc.partition_edge, nsub=sc.nsub, rxn_radius=sc.rxn_radius,
        verts=sc.verts, tris=sc.tris, space_steps=sc.space_steps, wall_class=sc.wall_class,
        rxn_ab=sc.rxn_ab, rxn_p=sc.rxn_p, mol_pos=sc.mol_pos, mol_species=sc.mol_species,
        mols=mols, disps=disps, draws=draws, results=res[:, :keep],
        info=info, wall_consts=wc_ref, wsp_counts=counts, wsp_list=lst)
    return res


def pathway_fixtures(ref64):
    """Reaction classes with several pathways (BNG::RxnClass cum_probs): a closed cube
    where A + B has three pathways and A + A two (kind-5 events record the pathway
    that fired), and test_bimolecular / which_unimolecular on injected draws over
    classes of 1-4 pathways, including the branch where the class's probability
    cannot be scaled enough (max_fixed_p >= scaling)."""
    rng = np.random.default_rng(20261204)
    sc = H.cube_scene(rng, n_mol=1500, nsub=12, partition_um=1.2)
    sc.rxn_ab = np.array([[0, 1], [0, 1], [0, 1], [0, 0], [0, 0]], np.uint32)
    sc.rxn_p = np.array([0.15, 0.25, 0.1, 0.3, 0.2])
    cases = [(m, d) for (m, d, _) in H.random_cases(rng, sc, 300, scale=2.0, near_wall_frac=0.3)]
    cases += partner_cases(rng, sc, 700)
    res = record_scene(ref64, rng, "pathways", sc, cases)
    fired = res[:, H.RES_HDR::H.EV_SIZE] == 5
    sides = res[:, H.RES_HDR + 2::H.EV_SIZE][fired]
    print("pathways", len(cases), "cases; pathways fired", np.unique(sides, return_counts=True))
    n = 800
    npw = rng.integers(1, 5, n)
    cum = np.zeros((n, 4))
    for i in range(n):
        p = rng.uniform(0, 0.6, npw[i]) * (4.0 if i % 5 == 0 else 1.0)
        cum[i, :npw[i]] = np.cumsum(p)
    scaling = rng.uniform(0, 1.5, n)
    scaling[::7] = 1.0
    U = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    U[::3] >>= 2
    bim = np.array([ref64.test_bimolecular_pw(cum[i, :npw[i]], scaling[i], U[i]) for i in range(n)], np.int32)
    m = 500
    unpw = rng.integers(1, 5, m)
    ucum = np.zeros((m, 4))
    for i in range(m):
        ucum[i, :unpw[i]] = np.cumsum(rng.uniform(0, 2e-3, unpw[i]))
    Uu = rng.integers(0, 2 ** 32, size=m, dtype=np.uint64).astype(np.uint32)
    Uu[:3] = [0, 1, 2 ** 32 - 1]
    uni = np.array([ref64.which_unimolecular(ucum[i, :unpw[i]], Uu[i]) for i in range(m)], np.int32)
    np.savez_compressed(HERE / "rxn_pathways.npz", cum=cum, npw=npw.astype(np.uint32), scaling=scaling, U=U,
                        bimol=bim, ucum=ucum, unpw=unpw.astype(np.uint32), Uu=Uu, unimol=uni)
    print("rxn pathways: bimolecular", np.unique(bim, return_counts=True), "unimolecular",
          np.unique(uni, return_counts=True))


def inside_fixtures(ref64):
    """Inside decisions on a closed non-convex object (the star-shaped sphere of
    H.star_scene, object 0, in a cube, object 1; both counted volumes):
    compute_counted_volume_for_pos (the counted-volume membership of a position) and
    is_point_inside_region_no_waypoints (the inside test of a release into a region),
    on points uniform in the cube and points within 1e-4-0.5 internal units of the
    object's faces, edges and vertices; and ReleaseEvent::release_ellipsoid_or_
    rectcuboid on injected random streams (sphere, cuboid, spherical shell)."""
    rng = np.random.default_rng(20261205)
    sc = H.star_scene(rng)
    h = ref64.scene(sc)
    h.set_objects(sc.obj, [1, 1])
    half = 60.0
    pts = [rng.uniform(-half, half, size=(3000, 3))]
    # near the star's surface: points of its triangles (vertices, edges, interiors) moved
    # along the face normal by a small signed offset
    sw = np.nonzero(sc.obj == 0)[0]
    tri = sc.tris[rng.choice(sw, 2000)]
    a, b, c = sc.verts[tri[:, 0]], sc.verts[tri[:, 1]], sc.verts[tri[:, 2]]
    u = rng.uniform(0, 1, (2000, 1))
    wv = rng.uniform(0, 1, (2000, 1))
    kind = rng.integers(0, 3, 2000)
    bary = np.where(kind[:, None] == 0, a, np.where(kind[:, None] == 1, a + (b - a) * u,
                                                     a + (b - a) * u * (1 - wv) + (c - a) * wv * (1 - u)))
    nrm = np.cross(b - a, c - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    off = np.exp(rng.uniform(np.log(1e-4), np.log(0.5), (2000, 1))) * rng.choice([-1.0, 1.0], (2000, 1))
    pts.append(bary + nrm * off)
    pts = np.concatenate(pts)
    cv = np.array([h.counted_volume_for_pos(p) for p in pts], np.uint32)
    reg = np.array([[h.inside_region(o, p) for o in (0, 1)] for p in pts], np.int32)
    # releases on injected streams
    n_rel = 60
    shapes = rng.integers(0, 3, n_rel).astype(np.int32)
    counts = rng.integers(1, 40, n_rel).astype(np.uint32)
    loc = rng.uniform(-30, 30, (n_rel, 3))
    dia = rng.uniform(1, 40, (n_rel, 3))
    nd = 512
    draws = rng.integers(0, 2 ** 32, size=(n_rel, nd), dtype=np.uint64).astype(np.uint32)
    rel_pos = np.zeros((n_rel, 40, 3))
    used = np.zeros(n_rel, np.int64)
    for k in range(n_rel):
        pos, u_ = ref64.release_ellipsoid_or_rectcuboid(int(shapes[k]), int(counts[k]), loc[k], dia[k], draws[k])
        assert u_ is not None
        rel_pos[k, :counts[k]] = pos
        used[k] = u_
    np.savez_compressed(
        HERE / "inside_star.npz",
        origin=sc.origin, partition_edge=sc.partition_edge, nsub=sc.nsub, rxn_radius=sc.rxn_radius, verts=sc.verts,
        tris=sc.tris, obj=sc.obj, points=pts, counted=cv, inside_region=reg, rel_shape=shapes, rel_n=counts,
        rel_loc=loc, rel_dia=dia, rel_draws=draws, rel_pos=rel_pos, rel_used=used)
    print("inside: points", len(pts), "in star", int(((cv & 1) > 0).sum()), "in cube", int(((cv & 2) > 0).sum()),
          "edge re-tries", int(((cv >> 31) & 1).sum()), "region tests", np.unique(reg, return_counts=True))


def star_fixture(ref64):
    """Diffusion cases on a closed non-convex object: the star-shaped sphere of
    H.star_scene (object 0, deep lobes, transparent to A, reflective to B) in a
    reflective cube, A + B -> C; random moves (half near walls) and moves aimed past a
    reacting partner."""
    rng = np.random.default_rng(20261207)
    sc = H.star_scene(rng, n_mol=1500, levels=3)
    sc.rxn_p = np.array([0.4])
    cases = [(m, d) for (m, d, _) in H.random_cases(rng, sc, 700, scale=3.0, near_wall_frac=0.5)]
    cases += partner_cases(rng, sc, 500)
    res = record_scene(ref64, rng, "star", sc, cases)
    kinds = np.unique(res[:, H.RES_HDR::H.EV_SIZE][res[:, H.RES_HDR::H.EV_SIZE] > 0], return_counts=True)
    print("star", len(cases), "cases, event kinds", dict(zip(kinds[0].astype(int).tolist(), kinds[1].tolist())))


def region_fixtures(ref64):
    """Releases into region expressions on H.regions_scene (star, box, small cube;
    closed objects 0-2): Region::initialize_volume_info_if_needed (object volumes),
    compute_region_expr_bounding_box, calculate_number_to_release by concentration, and
    ReleaseEvent::release_inside_regions on injected streams: a number of molecules into
    each expression of H.REGION_EXPRS, concentration releases into one object (exact)
    and into expressions (approximate count), and vacuums (negative numbers) of species
    0 from expressions (removed molecule indices)."""
    rng = np.random.default_rng(20261206)
    sc = H.regions_scene(rng)
    h = ref64.scene(sc)
    h.set_objects(sc.obj, [0, 0, 0])
    vol = np.array([h.region_volume(o) for o in range(3)])
    ex = H.REGION_EXPRS
    tok = np.full((len(ex), 15), 99, np.int32)
    for k, e in enumerate(ex):
        tok[k, :len(e)] = e
    ntok = np.array([len(e) for e in ex], np.int32)
    bbox = np.array([np.concatenate(h.region_expr_bbox(e)) for e in ex])
    dia = rng.uniform(1, 60, (40, 3))
    conc = np.exp(rng.uniform(np.log(1e-6), np.log(1e-2), 40))
    conc_n = np.array([ref64.number_from_concentration(d, c, 0.01) for d, c in zip(dia, conc)], np.int64)
    # releases: (expression, method, number, concentration)
    cases = [(k, 0, int(rng.integers(1, 60)), 0.0) for k in range(len(ex))]
    cases += [(1, 1, 0, 2e-6), (0, 1, 0, 3e-7)]                      # one object: exact count
    cases += [(3, 1, 0, 4e-7), (2, 1, 0, 1e-7), (6, 1, 0, 1e-7)]      # expressions: approximate
    cases += [(2, 0, -150, 0.0), (5, 0, -40, 0.0), (0, 0, -100000, 0.0), (4, 0, -7, 0.0)]  # vacuums
    nd = 40000
    draws = rng.integers(0, 2 ** 32, size=(len(cases), nd), dtype=np.uint64).astype(np.uint32)
    cap = 4000
    r_pos = np.zeros((len(cases), cap, 3))
    r_npos = np.zeros(len(cases), np.int64)
    r_rem = np.zeros((len(cases), cap), np.int64)
    r_nrem = np.zeros(len(cases), np.int64)
    r_used = np.zeros(len(cases), np.int64)
    r_computed = np.zeros(len(cases), np.int64)
    for c, (k, method, number, cc) in enumerate(cases):
        computed, pos, rem, used = h.release_inside_regions(ex[k], draws[c], number=number, species=0,
                                                            concentration=cc if method else None)
        assert used is not None and len(pos) <= cap and len(rem) <= cap, (c, used, len(pos))
        r_computed[c] = computed
        r_pos[c, :len(pos)] = pos
        r_npos[c] = len(pos)
        r_rem[c, :len(rem)] = rem
        r_nrem[c] = len(rem)
        r_used[c] = used
    # the vacuums' candidates in order: a vacuum of more than there are removes them all
    r_cand = np.zeros((len(cases), cap), np.int64)
    r_ncand = np.zeros(len(cases), np.int64)
    for c, (k, method, number, cc) in enumerate(cases):
        if number < 0:
            _, _, rem, _ = h.release_inside_regions(ex[k], draws[c], number=-(1 << 30), species=0)
            r_cand[c, :len(rem)] = rem
            r_ncand[c] = len(rem)
    draws = draws[:, :int(r_used.max()) + 16]  # the draws the reference took, and a few more
    case_arr = np.array([[k, m, n] for (k, m, n, _) in cases], np.int64)
    case_conc = np.array([cc for (_, _, _, cc) in cases])
    np.savez_compressed(
        HERE / "regions.npz",
        origin=sc.origin, partition_edge=sc.partition_edge, nsub=sc.nsub, rxn_radius=sc.rxn_radius, verts=sc.verts,
        tris=sc.tris, obj=sc.obj, mol_pos=sc.mol_pos, mol_species=sc.mol_species, volumes=vol, expr=tok,
        n_expr=ntok, bbox=bbox, conc_dia=dia, conc=conc, conc_n=conc_n, cases=case_arr, case_conc=case_conc,
        draws=draws, computed=r_computed, pos=r_pos, n_pos=r_npos, removed=r_rem, n_removed=r_nrem, used=r_used,
        candidates=r_cand, n_candidates=r_ncand)
    print("regions: volumes", vol, "placed", r_npos.tolist(), "removed", r_nrem.tolist())


def main():
    ref64 = H.reference(64)
    if ref64 is None:
        raise SystemExit("oracle/_ref/libmcell_ref64.so missing: run python oracle/ref/build_ref.py")
    if sys.argv[1:] == ["regions"]:
        region_fixtures(ref64)
        return
    if sys.argv[1:] == ["star"]:
        star_fixture(ref64)
        return
    rng = np.random.default_rng(20261203)
    for name, sc in scenes(rng).items():
        cases = []
        if name == "cube":
            cases += add_edge_molecules(sc)
        cases += [(m, d) for (m, d, _) in H.random_cases(rng, sc, 700, scale=2.0, near_wall_frac=0.4)]
        cases += partner_cases(rng, sc, 500)
        res = record_scene(ref64, rng, name, sc, cases)
        kinds = np.unique(res[:, H.RES_HDR::H.EV_SIZE][res[:, H.RES_HDR::H.EV_SIZE] > 0], return_counts=True)
        print(name, len(cases), "cases, event kinds", dict(zip(kinds[0].astype(int).tolist(), kinds[1].tolist())),
              "status", np.unique(res[:, 0], return_counts=True))
    # reaction tests on injected uniforms
    P = np.concatenate([rng.uniform(0, 1, 400), rng.uniform(0, 3, 100), [0.0, 1.0, 2.0, 0.0368]])
    S = np.concatenate([rng.uniform(0, 1.5, 400), rng.uniform(0, 3, 100), [1.0, 1.0, 1.0, 1.0]])
    U = rng.integers(0, 2 ** 32, size=len(P), dtype=np.uint64).astype(np.uint32)
    tb = np.array([ref64.test_bimolecular(p, s, u) for p, s, u in zip(P, S, U)], np.int32)
    K = rng.uniform(0, 2e-3, 300)
    Uu = rng.integers(0, 2 ** 32, size=len(K), dtype=np.uint64).astype(np.uint32)
    Uu[:3] = [0, 1, 2 ** 32 - 1]
    tu = np.array([ref64.time_of_unimol(k, u) for k, u in zip(K, Uu)])
    # the reference's ISAAC64 + ziggurat Gaussian stream (distribution reference)
    import ctypes
    g = np.zeros(20000)
    ref64.lib.ref_rng_gauss(ctypes.c_ulonglong(1), ctypes.c_uint(len(g)), H.ptr(g))
    np.savez_compressed(HERE / "rxn_tests.npz", P=P, S=S, U=U, bimol=tb, K=K, Uu=Uu, unimol=tu, ref_gauss=g)
    print("rxn tests", (tb >= 0).sum(), "fired of", len(tb))
    pathway_fixtures(ref64)
    inside_fixtures(ref64)
    region_fixtures(ref64)
    star_fixture(ref64)


if __name__ == "__main__":
    main()
