"""Test harness: scenes, and ctypes bindings to the two CPU checkers.

- the oracle port (oracle/_build/libmcell_oracle.so, built everywhere by build())
- the reference's own routines (oracle/_ref/libmcell_ref{64,32}.so, built only
  where the reference sources exist, i.e. not on the GPU host)

Both expose the same scene / case entry points (prefix orc_ / ref_). Results of
one diffusion case are float64 arrays of RES_SIZE (layout in oracle/mcell_oracle.h).
"""
from __future__ import annotations

import ctypes
import math
import os
import sys
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional

import numpy as np

from mcell_gb300 import conversion, geometry

ROOT = Path(__file__).resolve().parent.parent
RES_HDR, EV_SIZE, EV_MAX = 9, 8, 32
RES_SIZE = RES_HDR + EV_SIZE * EV_MAX

_vp = ctypes.c_void_p
_d = ctypes.c_double
_u = ctypes.c_uint


def ptr(a):
    return a.ctypes.data_as(_vp)


@dataclass
class Scene:
    origin: np.ndarray
    partition_edge: float
    nsub: int
    rxn_radius: float
    verts: np.ndarray             # float64 [nv, 3] internal units
    tris: np.ndarray              # uint32 [nw, 3]
    space_steps: np.ndarray       # float64 [nspecies]
    wall_class: np.ndarray        # uint8 [nw, nspecies]
    rxn_ab: np.ndarray            # uint32 [nrxn, 2]
    rxn_p: np.ndarray             # float64 [nrxn]
    mol_pos: np.ndarray           # float64 [nmol, 3]
    mol_species: np.ndarray       # uint32 [nmol]

    def args(self):
        o = np.ascontiguousarray(self.origin, np.float64)
        keep = [o, np.ascontiguousarray(self.verts, np.float64), np.ascontiguousarray(self.tris, np.uint32),
                np.ascontiguousarray(self.space_steps, np.float64),
                np.ascontiguousarray(self.wall_class, np.uint8),
                np.ascontiguousarray(self.rxn_ab, np.uint32).reshape(-1),
                np.ascontiguousarray(self.rxn_p, np.float64),
                np.ascontiguousarray(self.mol_pos, np.float64), np.ascontiguousarray(self.mol_species, np.uint32)]
        self._keep = keep
        return (ptr(keep[0]), _d(self.partition_edge), _u(self.nsub), _d(self.rxn_radius),
                _u(len(self.verts)), ptr(keep[1]), _u(len(self.tris)), ptr(keep[2]),
                _u(len(self.space_steps)), ptr(keep[3]), ptr(keep[4]),
                _u(len(self.rxn_p)), ptr(keep[5]), ptr(keep[6]),
                _u(len(self.mol_species)), ptr(keep[7]), ptr(keep[8]))


class Checker:
    """One of the two CPU checkers (oracle port or reference routines)."""

    def __init__(self, path: Path, prefix: str):
        self.lib = ctypes.CDLL(str(path))
        self.p = prefix
        f = self.fn("scene_new")
        f.restype = _vp
        self.fn("subpart_index").restype = _u
        self.fn("scene_walls_in_subparts").restype = _u
        self.fn("test_bimolecular").restype = ctypes.c_int
        self.fn("test_bimolecular_pw").restype = ctypes.c_int
        self.fn("which_unimolecular").restype = ctypes.c_int
        self.fn("time_of_unimol").restype = _d

    def fn(self, name):
        return getattr(self.lib, f"{self.p}_{name}")

    def scene(self, sc: Scene):
        h = _vp(self.fn("scene_new")(*sc.args()))
        return _Handle(self, h)

    def test_bimolecular(self, p, scaling, draw):
        return self.fn("test_bimolecular")(_d(p), _d(scaling), _u(draw))

    def time_of_unimol(self, k, draw):
        return self.fn("time_of_unimol")(_d(k), _u(draw))

    def release_ellipsoid_or_rectcuboid(self, shape, n, location, diameter, draws):
        """Positions [n, 3] of a release (shape 0 sphere, 1 cuboid, 2 shell) drawing from
        `draws`, and the draws used (None if they ran out)."""
        out = np.zeros((n, 3))
        loc = np.ascontiguousarray(location, np.float64)
        dia = np.ascontiguousarray(diameter, np.float64)
        dr = np.ascontiguousarray(draws, np.uint32)
        f = self.fn("release_ellipsoid_or_rectcuboid")
        f.restype = _u
        used = f(ctypes.c_int(shape), _u(n), ptr(loc), ptr(dia), ptr(dr), _u(len(dr)), ptr(out))
        return out, (None if used == 0xFFFFFFFF else int(used))

    def test_bimolecular_pw(self, cum, scaling, draw):
        """test_bimolecular over a class of len(cum) pathways: pathway index, < 0 = none."""
        c = np.ascontiguousarray(cum, np.float64)
        return self.fn("test_bimolecular_pw")(ptr(c), _u(len(c)), _d(scaling), _u(draw))

    def which_unimolecular(self, cum, draw):
        c = np.ascontiguousarray(cum, np.float64)
        return self.fn("which_unimolecular")(ptr(c), _u(len(c)), _u(draw))

    def number_from_concentration(self, diameter, concentration, length_unit_um):
        """ReleaseEvent::calculate_number_to_release for a spherical concentration release."""
        d = np.ascontiguousarray(diameter, np.float64)
        f = self.fn("number_from_concentration")
        f.restype = _u
        return f(ptr(d), _d(concentration), _d(length_unit_um))


class _Handle:
    def __init__(self, chk: Checker, h):
        self.c, self.h = chk, h

    def __del__(self):
        try:
            self.c.fn("scene_free")(self.h)
        except Exception:
            pass

    def info(self):
        out = np.zeros(7)
        self.c.fn("scene_info")(self.h, ptr(out))
        return out

    def wall_consts(self, nw):
        out = np.zeros((nw, 14))
        self.c.fn("scene_wall_consts")(self.h, ptr(out))
        return out

    def walls_in_subparts(self, nsub3, cap=1 << 22):
        counts = np.zeros(nsub3, np.uint32)
        lst = np.zeros(cap, np.uint32)
        n = self.c.fn("scene_walls_in_subparts")(self.h, ptr(counts), ptr(lst), _u(cap))
        return counts, lst[:n]

    def subpart_index(self, pos):
        p = np.ascontiguousarray(pos, np.float64)
        return self.c.fn("subpart_index")(self.h, ptr(p))

    def exact_disk(self, loc, mv, moving, target):
        """exact_disk at loc for molecule `moving` (move mv) against molecule `target`:
        the unoccluded fraction of the reaction disk, or < 0 when a wall blocks it."""
        f = self.c.fn("exact_disk")
        f.restype = _d
        l = np.ascontiguousarray(loc, np.float64)
        m = np.ascontiguousarray(mv, np.float64)
        return f(self.h, ptr(l), ptr(m), _u(moving), _u(target))

    def set_objects(self, object_of_wall, counted):
        """Geometry objects: the object index of each wall; counted[k] marks counted volumes."""
        ow = np.ascontiguousarray(object_of_wall, np.uint32)
        cn = np.ascontiguousarray(counted, np.uint8)
        self.c.fn("scene_set_objects")(self.h, _u(len(cn)), ptr(ow), ptr(cn))

    def counted_volume_for_pos(self, pos):
        """Bit mask of the counted objects containing pos; bit 31: the ray met an edge."""
        p = np.ascontiguousarray(pos, np.float64)
        f = self.c.fn("counted_volume_for_pos")
        f.restype = _u
        return f(self.h, ptr(p))

    def inside_region(self, obj, pos):
        """0 outside / 1 inside the closed region of object obj; 2: the ray met an edge."""
        p = np.ascontiguousarray(pos, np.float64)
        f = self.c.fn("inside_region")
        f.restype = ctypes.c_int
        return f(self.h, _u(obj), ptr(p))

    def region_volume(self, obj):
        """Region::initialize_volume_info_if_needed: the closed object's volume."""
        f = self.c.fn("region_volume")
        f.restype = _d
        return f(self.h, _u(obj))

    def region_expr_bbox(self, tokens):
        """compute_region_expr_bounding_box of a postfix program (objects, -1 union,
        -2 intersection, -3 difference): (llf, urb)."""
        t = np.ascontiguousarray(tokens, np.int32)
        lo, hi = np.zeros(3), np.zeros(3)
        self.c.fn("region_expr_bbox")(self.h, ptr(t), _u(len(t)), ptr(lo), ptr(hi))
        return lo, hi

    def release_inside_regions(self, tokens, draws, number=0, species=0, concentration=None, length_unit_um=0.01,
                               cap=100000):
        """ReleaseEvent::release_inside_regions on injected draws: (computed number,
        positions, removed molecule indices, draws used or None)."""
        t = np.ascontiguousarray(tokens, np.int32)
        dr = np.ascontiguousarray(draws, np.uint32)
        pos = np.zeros((cap, 3))
        rem = np.zeros(cap, np.uint32)
        n_pos, n_rem, used = _u(), _u(), _u()
        f = self.c.fn("release_inside_regions")
        f.restype = ctypes.c_int
        computed = f(self.h, ptr(t), _u(len(t)), ctypes.c_int(0 if concentration is None else 1),
                     ctypes.c_int(number), _u(species), _d(concentration or 0.0), _d(length_unit_um), ptr(dr),
                     _u(len(dr)), ptr(pos), _u(cap), ctypes.byref(n_pos), ptr(rem), ctypes.byref(n_rem),
                     ctypes.byref(used))
        return (computed, pos[:n_pos.value], rem[:n_rem.value], None if used.value == 0xFFFFFFFF else used.value)

    def diffuse_case(self, mol, disp, draws, r_rate_factor=1.0, t_steps=1.0):
        out = np.zeros(RES_SIZE)
        d = np.ascontiguousarray(disp, np.float64)
        dr = np.ascontiguousarray(draws, np.uint32)
        self.c.fn("diffuse_case")(self.h, _u(mol), ptr(d), ptr(dr), _u(len(dr)), _d(r_rate_factor),
                                  _d(t_steps), ptr(out))
        return out


def oracle_path() -> Path:
    return ROOT / "oracle" / "_build" / "libmcell_oracle.so"


def ref_path(bits=64) -> Path:
    return ROOT / "oracle" / "_ref" / f"libmcell_ref{bits}.so"


def oracle() -> Checker:
    return Checker(oracle_path(), "orc")


def reference(bits=64) -> Optional[Checker]:
    p = ref_path(bits)
    if not p.exists():
        return None
    return Checker(p, "ref")


# ------------------------------------------------------------------ scenes

def cube_scene(rng: np.random.Generator, n_mol=400, edge_um=1.0, nsub=12, partition_um=1.2,
               p_rxn=0.0368, classes=None) -> Scene:
    """Closed reflective cube (the Model API's create_box) with A (0), B (1), C (2)."""
    lu = conversion.length_unit_um()
    v, w = geometry.create_box(edge_dimension=edge_um)
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=partition_um,
                                      subpartition_dimension_um=partition_um / nsub)
    verts = v / lu
    half = edge_um / 2 / lu
    pos = rng.uniform(-half, half, size=(n_mol, 3))
    sp = rng.integers(0, 2, size=n_mol).astype(np.uint32)
    wc = np.zeros((len(w), 3), np.uint8)
    if classes is not None:
        wc[:] = classes
    return Scene(np.array(lay.origin), lay.edge, lay.nsub, conversion.default_rxn_radius_um() / lu,
                 verts, w, np.array([2.0, 2.0, 1.414213562373095]), wc,
                 np.array([[0, 1]], np.uint32), np.array([p_rxn]), pos, sp)


def sphere_in_cube_scene(rng: np.random.Generator, levels=2, n_mol=400, radius_um=1.0, cube_um=2.5,
                         nsub=None, transparent_a=True, p_rxn=0.0368) -> Scene:
    """Icosphere inside a reflective cube; sphere transparent to A (config of the large model)."""
    lu = conversion.length_unit_um()
    sv, sw = geometry.create_icosphere(radius_um, levels)
    bv, bw = geometry.create_box(edge_dimension=cube_um)
    v, w, obj = geometry.merge_meshes((sv, sw), (bv, bw))
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=cube_um + 0.2,
                                      subpartition_dimension_um=0.1)
    if nsub is not None:
        lay = conversion.PartitionLayout(lay.origin, lay.edge, nsub)
    wc = np.zeros((len(w), 3), np.uint8)
    if transparent_a:
        wc[obj == 0, 0] = 1
    half = cube_um / 2 / lu
    pos = rng.uniform(-half, half, size=(n_mol, 3))
    sp = rng.integers(0, 2, size=n_mol).astype(np.uint32)
    return Scene(np.array(lay.origin), lay.edge, lay.nsub, conversion.default_rxn_radius_um() / lu,
                 v / lu, w, np.array([2.0, 2.0, 1.414213562373095]), wc,
                 np.array([[0, 1]], np.uint32), np.array([p_rxn]), pos, sp)


def random_cases(rng: np.random.Generator, sc: Scene, n_cases: int, scale=2.0, ndraws=64, near_wall_frac=0.3):
    """Random diffusion cases: (molecule index, displacement, draws). A fraction starts near walls."""
    cases = []
    nm = len(sc.mol_species)
    for _ in range(n_cases):
        mol = int(rng.integers(0, nm))
        disp = rng.normal(0.0, scale * 0.7071067811865476, size=3)
        if rng.random() < near_wall_frac:
            disp *= rng.uniform(2, 20)
        draws = rng.integers(0, 2 ** 32, size=ndraws, dtype=np.uint64).astype(np.uint32)
        cases.append((mol, disp, draws))
    return cases


def engine_from_scene(sc: Scene, precision="fp64", seed=1, capacity=0):
    """GPU engine holding the scene's mesh, reactions and molecules (ids = scene order)."""
    from mcell_gb300._native import Engine
    nsp = len(sc.space_steps)
    e = Engine(precision, sc.origin, sc.partition_edge, sc.nsub, sc.rxn_radius, nsp, seed=seed, capacity=capacity)
    e.set_species(sc.space_steps)
    e.upload_mesh(sc.verts, sc.tris, sc.wall_class.reshape(len(sc.tris), nsp))
    for (a, b), p in zip(np.asarray(sc.rxn_ab).reshape(-1, 2), sc.rxn_p):
        e.add_bimol_rxn(int(a), int(b), float(p))
    e.add_molecules(sc.mol_pos, sc.mol_species)
    e.prepare()
    return e


def edge_cases(sc: Scene):
    """Hand-made cases for the closed cube of edge 100 internal units (create_box order):
    hits on a face diagonal (REDO), a cube vertex, a cube edge, a molecule on a wall
    plane moving along it and away from it, corner multi-bounces."""
    P = [
        ((40.0, 10.0, 10.0), (20.0, 0.0, 0.0)),     # x=+50 face, on the y==z diagonal
        ((40.0, 40.0, 40.0), (20.0, 20.0, 20.0)),   # straight into the (50,50,50) vertex
        ((40.0, 40.0, 0.0), (20.0, 20.0, 0.0)),     # into the x=y=50 edge
        ((-40.0, 5.0, -5.0), (-20.0, 0.0, 0.0)),    # x=-50 face
        ((0.0, 0.0, 49.0), (0.0, 0.0, 3.0)),        # z=+50 face, perpendicular
        ((45.0, 45.0, 45.0), (15.0, 12.0, 9.0)),    # corner, several reflections
        ((-45.0, -45.0, 45.0), (-30.0, -25.0, 20.0)),
        ((0.0, 0.0, 0.0), (170.0, 130.0, 110.0)),   # long ray, many reflections
        ((10.0, -20.0, 30.0), (1e-3, 2e-3, -1e-3)), # tiny step
        ((49.999999, 1.0, 2.0), (0.5, 0.1, 0.0)),   # starts just below the wall
        ((-30.0, 20.0, 49.0), (0.0, 0.0, 1.0)),     # lands exactly on the wall plane
    ]
    return P


GOLDEN = ROOT / "tests" / "golden"
GOLDEN_SCENES = ["cube", "cube_dense", "cube_classes", "sphere", "pathways", "star"]


def star_scene(rng, n_mol=200, levels=3):
    """A closed non-convex object (geometry.create_star_sphere, radius 0.45 um, object 0,
    transparent to A) in a reflective 1.2 um cube (object 1); objects per wall in .obj."""
    lu = conversion.length_unit_um()
    sv, sw = geometry.create_star_sphere(0.45, levels)
    bv, bw = geometry.create_box(edge_dimension=1.2)
    v, w, obj = geometry.merge_meshes((sv, sw), (bv, bw))
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=1.3, subpartition_dimension_um=0.1)
    wc = np.zeros((len(w), 3), np.uint8)
    wc[obj == 0, 0] = 1
    half = 0.6 / lu
    pos = rng.uniform(-half, half, size=(n_mol, 3))
    sp = rng.integers(0, 2, size=n_mol).astype(np.uint32)
    sc = Scene(np.array(lay.origin), lay.edge, lay.nsub, conversion.default_rxn_radius_um() / lu, v / lu, w,
               np.array([2.0, 2.0, 1.414213562373095]), wc, np.array([[0, 1]], np.uint32), np.array([0.0]), pos, sp)
    sc.obj = np.asarray(obj, np.uint32)
    return sc


def regions_scene(rng, n_mol=3000):
    """Three closed objects for region releases: the non-convex star (object 0, radius
    0.45 um), the 1.2 um reflective box (object 1) and a 0.4 um cube centred at
    (0.2531, 0.2017, 0.1493) um (object 2) that overlaps the star; molecules uniform in the box."""
    lu = conversion.length_unit_um()
    sv, sw = geometry.create_star_sphere(0.45, 3)
    bv, bw = geometry.create_box(edge_dimension=1.2)
    cv, cw = geometry.create_box(edge_dimension=0.4)
    cv = cv + np.array([0.2531, 0.2017, 0.1493])
    v, w, obj = geometry.merge_meshes((sv, sw), (bv, bw), (cv, cw))
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=1.3, subpartition_dimension_um=0.1)
    wc = np.zeros((len(w), 3), np.uint8)
    half = 0.6 / lu
    pos = rng.uniform(-half, half, size=(n_mol, 3))
    sp = rng.integers(0, 2, size=n_mol).astype(np.uint32)
    sc = Scene(np.array(lay.origin), lay.edge, lay.nsub, conversion.default_rxn_radius_um() / lu, v / lu, w,
               np.array([2.0, 2.0, 1.414213562373095]), wc, np.array([[0, 1]], np.uint32), np.array([0.0]), pos, sp)
    sc.obj = np.asarray(obj, np.uint32)
    return sc


# region expressions of the region fixture (postfix; -1 union, -2 intersection, -3 difference)
REGION_EXPRS = [[0], [2], [1, 0, -3], [0, 2, -1], [0, 2, -2], [2, 0, -3], [1, 0, -3, 2, -1]]


def load_golden(name):
    """(Scene, cases dict) of a golden fixture made by tests/golden/make_golden.py."""
    z = np.load(GOLDEN / f"diffuse_{name}.npz")
    sc = Scene(z["origin"], float(z["partition_edge"]), int(z["nsub"]), float(z["rxn_radius"]), z["verts"],
               z["tris"], z["space_steps"], z["wall_class"], z["rxn_ab"], z["rxn_p"], z["mol_pos"],
               z["mol_species"])
    return sc, {k: z[k] for k in ("mols", "disps", "draws", "results", "info", "wall_consts", "wsp_counts",
                                  "wsp_list")}


def compare_results(got, want, rel=0.0, scene: Optional[Scene] = None):
    """Compares case results: integer fields exactly; times / positions exactly (rel=0)
    or within a relative tolerance. Returns the list of mismatching case indices.
    A molecule that ends outside the partition (the reference's fatal escape) has no
    meaningful subpartition index, so with `scene` given that field is skipped for it."""
    bad = []
    k = want.shape[1]
    for c in range(len(want)):
        g, w = got[c, :k], want[c, :k]
        n = int(w[6])
        ints = [0, 5, 6] + [RES_HDR + e * EV_SIZE + f for e in range(min(n, EV_MAX)) for f in (0, 1, 2)]
        escaped = False
        if scene is not None:
            lo = np.asarray(scene.origin)
            escaped = bool(np.any(w[1:4] < lo) or np.any(w[1:4] >= lo + scene.partition_edge))
        if not escaped:
            ints.append(4)
        if not np.array_equal(g[ints], w[ints]):
            bad.append(c)
            continue
        fl = [i for i in range(k) if i not in ints and i != 4]
        if rel == 0.0:
            ok = np.array_equal(g[fl], w[fl])
        else:
            ok = np.allclose(g[fl], w[fl], rtol=rel, atol=rel)
        if not ok:
            bad.append(c)
    return bad


# ------------------------------------------------------------------ engines with chemistry

sys.path.insert(0, str(ROOT))
from oracle.oracle_py import OracleEngine, make_oracle_engine  # noqa: E402,F401


def make_gpu_engine(sc: Scene, precision="fp64", bimol=(), unimol=(), seed=1, capacity=0):
    """GPU engine with explicit chemistry: bimol [(a, b, p, (p0, p1))], unimol [(a, k, (p0, p1))]."""
    from mcell_gb300._native import Engine
    nsp = len(sc.space_steps)
    e = Engine(precision, sc.origin, sc.partition_edge, sc.nsub, sc.rxn_radius, nsp, seed=seed, capacity=capacity)
    e.set_species(sc.space_steps)
    e.upload_mesh(sc.verts, sc.tris, np.asarray(sc.wall_class).reshape(len(sc.tris), nsp))
    for a, b, p, pr in bimol:
        e.add_bimol_rxn(a, b, p, pr)
    for a, k, pr in unimol:
        e.add_unimol_rxn(a, k, pr)
    e.add_molecules(sc.mol_pos, sc.mol_species)
    e.prepare()
    return e
