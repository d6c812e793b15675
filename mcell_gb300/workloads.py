"""Synthetic models of the benchmark configurations, in internal units.

Each builder returns a Model description (plain arrays) that the engine and the
oracle both accept. Inputs are seeded synthetic data with the shapes, sizes
and parameters of the configurations (no public dataset is involved):

- closed_cube: a reflective 1 um cube (the Model API's create_box) with A and B
  uniformly inside, D_A = D_B = 1e-6 cm^2/s, C with 5e-7, A + B -> C at
  1e8 M^-1 s^-1, dt = 1 us, subpartitions of 0.1 um.
- replica_models: the batching / serving distribution of independent models
  (cubes of 0.5-3 um, optional icospheres of level 2-5, 1k-200k molecules,
  k from 1e6 to 1e9 M^-1 s^-1).
- bumpy_tube: the precision stress model (10M molecules in a 200k-triangle
  bumpy tube, 5% within 1 nm of mesh edges and vertices, dt = 0.1 us).
- sphere_in_cube: an icosphere of radius 1 um (20,480 triangles at 5 subdivision
  levels) transparent to A and reflective to B and C, centred in a reflective
  2.5 um cube; A and B 1:1 uniformly in the cube; A + B -> C at 1e8 M^-1 s^-1,
  C -> 0 at 1e3 s^-1; dt = 1 us; positions in fp32 on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

from . import conversion, geometry

SPECIES = ("A", "B", "C")


@dataclass
class Model:
    name: str
    origin: Tuple[float, float, float]
    partition_edge: float
    nsub: int
    rxn_radius: float
    verts: np.ndarray
    walls: np.ndarray
    wall_class: np.ndarray          # [n_walls, n_species] 0 reflect, 1 transparent, 2 absorptive
    space_steps: np.ndarray
    bimol: List[tuple] = field(default_factory=list)   # (a, b, max_fixed_p, (p0, p1))
    unimol: List[tuple] = field(default_factory=list)  # (a, k_tot, (p0, p1))
    pos: np.ndarray = None
    species: np.ndarray = None
    time_step_s: float = 1e-6

    @property
    def n_species(self):
        return len(self.space_steps)


def _chemistry(dt, lu, R_um, k_bimol=1e8, k_unimol=None):
    d = (1e-6, 1e-6, 5e-7)
    steps = np.array([conversion.space_step(x, dt, lu) for x in d])
    p = conversion.bimol_probability(k_bimol, steps[0], steps[1], R_um, dt, lu)
    bimol = [(0, 1, p, (2, -1))]
    unimol = [] if k_unimol is None else [(2, conversion.unimol_k_tot(k_unimol, dt), (-1, -1))]
    return steps, bimol, unimol


def closed_cube(n_per_species=5000, seed=1, edge_um=1.0, partition_um=1.2, subpart_um=0.1, dt=1e-6) -> Model:
    lu = conversion.length_unit_um()
    R_um = conversion.default_rxn_radius_um()
    v, w = geometry.create_box(edge_dimension=edge_um)
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=partition_um,
                                      subpartition_dimension_um=subpart_um)
    steps, bimol, unimol = _chemistry(dt, lu, R_um)
    rng = np.random.default_rng(seed)
    half = edge_um / 2 / lu
    n = 2 * n_per_species
    pos = rng.uniform(-half, half, size=(n, 3))
    sp = np.repeat(np.array([0, 1], np.uint32), n_per_species)
    return Model("closed_cube", lay.origin, lay.edge, lay.nsub, R_um / lu, v / lu, w,
                 np.zeros((len(w), 3), np.uint8), steps, bimol, unimol, pos, sp, dt)


def sphere_in_cube(n_mol=1_000_000, seed=1, levels=5, radius_um=1.0, cube_um=2.5, partition_um=2.6,
                   subpart_um=0.1, dt=1e-6) -> Model:
    lu = conversion.length_unit_um()
    R_um = conversion.default_rxn_radius_um()
    sv, sw = geometry.create_icosphere(radius_um, levels)
    bv, bw = geometry.create_box(edge_dimension=cube_um)
    v, w, obj = geometry.merge_meshes((sv, sw), (bv, bw))
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=partition_um,
                                      subpartition_dimension_um=subpart_um)
    wc = np.zeros((len(w), 3), np.uint8)
    wc[obj == 0, 0] = 1  # the sphere is transparent to A
    steps, bimol, unimol = _chemistry(dt, lu, R_um, k_unimol=1e3)
    rng = np.random.default_rng(seed)
    half = cube_um / 2 / lu
    pos = rng.uniform(-half, half, size=(n_mol, 3))
    sp = (np.arange(n_mol) % 2).astype(np.uint32)
    return Model("sphere_in_cube", lay.origin, lay.edge, lay.nsub, R_um / lu, v / lu, w, wc, steps, bimol, unimol,
                 pos, sp, dt)


def bumpy_tube(n_mol=10_000_000, seed=1, length_um=10.0, radius_um=0.2, bump_um=0.05, n_theta=200, n_z=500,
               near_edge_frac=0.05, near_nm=1.0, dt=1e-7, subparts_per_edge=300) -> Model:
    """Precision stress: the bumpy tube of geometry.create_bumpy_tube (reflective,
    200,400 triangles at the defaults) holding n_mol molecules, A:B 1:1; a fraction
    near_edge_frac of them sits within near_nm nm of a mesh edge or vertex (moved
    inwards from a random point of a random side edge, or from a random side
    vertex, away from the two rows of triangles that meet the end caps), the rest
    uniform inside (at least 2 nm from the analytic surface, so
    inside the triangulated one). A + B -> C at 1e8 M^-1 s^-1, D = 1e-6 cm^2/s
    (C: 5e-7), dt = 1e-7 s. The partition is the cube around the tube with
    subparts_per_edge subpartitions per edge."""
    lu = conversion.length_unit_um()
    R_um = conversion.default_rxn_radius_um()
    waves = 2.0 * length_um  # 20 axial waves over the 10 um tube
    v, w = geometry.create_bumpy_tube(radius_um, length_um, bump_um, n_theta, n_z, axial_waves=waves)
    edge = length_um + 0.2
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=edge,
                                      subpartition_dimension_um=edge / subparts_per_edge)
    steps, bimol, unimol = _chemistry(dt, lu, R_um)
    rng = np.random.default_rng(seed)
    n_near = int(round(n_mol * near_edge_frac))
    n_uni = n_mol - n_near
    # uniform inside: z, theta uniform, r^2 uniform below the surface radius - 2 nm
    z = rng.uniform(-length_um / 2 + 0.002, length_um / 2 - 0.002, n_uni)
    th = rng.uniform(0, 2 * np.pi, n_uni)
    rs = radius_um + bump_um * np.sin(2 * np.pi * waves * (z + length_um / 2) / length_um) * np.sin(4 * th) - 0.002
    r = rs * np.sqrt(rng.uniform(0, 1, n_uni))
    uni = np.stack([r * np.cos(th), r * np.sin(th), z], axis=1)
    # near edges / vertices of the side: a point of a side edge (or a side vertex)
    # moved towards the axis by up to near_nm, plus a jitter of the same size along it
    n_side = n_theta * (n_z + 1)
    half = n_near // 2
    # side triangles come first, row by row; the first and last rows are left out: their
    # edges reach the end rings, where the surface narrows towards the cap within one
    # row, and a point there kept below the cap by the clip below can lie outside it
    sw = rng.integers(2 * n_theta, 2 * n_theta * (n_z - 1), half)
    k = rng.integers(0, 3, half)
    a = v[w[sw, k]]
    b = v[w[sw, (k + 1) % 3]]
    p_edge = a + (b - a) * rng.uniform(0, 1, (half, 1))
    p_vert = v[rng.integers(n_theta, n_side - n_theta, n_near - half)]  # not the end rings
    near = np.concatenate([p_edge, p_vert])
    inward = -near.copy()
    inward[:, 2] = 0
    inward /= np.linalg.norm(inward, axis=1, keepdims=True)
    dist = rng.uniform(1e-3, near_nm, len(near)) * 1e-3  # um
    jitter = rng.normal(size=near.shape)
    jitter -= (jitter * inward).sum(1, keepdims=True) * inward
    jitter *= (rng.uniform(0, 0.5, (len(near), 1)) * dist[:, None]) / np.linalg.norm(jitter, axis=1, keepdims=True)
    near = near + inward * dist[:, None] + jitter
    near[:, 2] = np.clip(near[:, 2], -length_um / 2 + 0.002, length_um / 2 - 0.002)
    pos = np.concatenate([uni, near]) / lu
    sp = (np.arange(n_mol) % 2).astype(np.uint32)
    wc = np.zeros((len(w), 3), np.uint8)
    return Model("bumpy_tube", lay.origin, lay.edge, lay.nsub, R_um / lu, v / lu, w, wc, steps, bimol, unimol,
                 pos, sp, dt)


def replica_models(n_replicas=256, seed=7, n_range=(1_000, 200_000), edge_range_um=(0.5, 3.0),
                   k_range=(1e6, 1e9), levels=(2, 5), sphere_fraction=0.5, dt=1e-6):
    """Independent models for batching and serving: reflective cubes of edge
    log-uniform in edge_range_um, half of them (sphere_fraction) holding an
    icosphere of radius 0.4 x edge and level uniform in levels (transparent to A,
    reflective to B and C); molecule counts log-uniform in n_range (A:B 1:1,
    uniform in the cube); A + B -> C with k log-uniform in k_range M^-1 s^-1,
    C -> 0 at 1e3 s^-1; D = 1e-6 cm^2/s (C: 5e-7); subpartitions of 0.1 um."""
    lu = conversion.length_unit_um()
    R_um = conversion.default_rxn_radius_um()
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_replicas):
        edge = float(np.exp(rng.uniform(np.log(edge_range_um[0]), np.log(edge_range_um[1]))))
        n_mol = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        k = float(np.exp(rng.uniform(np.log(k_range[0]), np.log(k_range[1]))))
        bv, bw = geometry.create_box(edge_dimension=edge)
        if rng.uniform() < sphere_fraction:
            level = int(rng.integers(levels[0], levels[1] + 1))
            sv, sw = geometry.create_icosphere(0.4 * edge, level)
            v, w, obj = geometry.merge_meshes((sv, sw), (bv, bw))
            wc = np.zeros((len(w), 3), np.uint8)
            wc[obj == 0, 0] = 1
        else:
            v, w = bv, bw
            wc = np.zeros((len(w), 3), np.uint8)
        lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=edge + 0.1,
                                          subpartition_dimension_um=0.1)
        steps, bimol, unimol = _chemistry(dt, lu, R_um, k_bimol=k, k_unimol=1e3)
        half = edge / 2 / lu
        pos = rng.uniform(-half, half, size=(n_mol, 3))
        sp = (np.arange(n_mol) % 2).astype(np.uint32)
        out.append(Model(f"replica{r}", lay.origin, lay.edge, lay.nsub, R_um / lu, v / lu, w, wc, steps, bimol,
                         unimol, pos, sp, dt))
    return out


def model_handle(model: Model, precision="fp32", seed=1, capacity=0, with_molecules=True):
    """An engine handle holding the model's description, not yet prepared (the
    form a batch takes models in)."""
    from ._native import Engine

    e = Engine(precision, model.origin, model.partition_edge, model.nsub, model.rxn_radius, model.n_species,
               seed=seed, capacity=capacity or int(len(model.species) * 1.5) + 1024)
    e.set_species(model.space_steps)
    e.upload_mesh(model.verts, model.walls, model.wall_class)
    for a, b, p, pr in model.bimol:
        e.add_bimol_rxn(a, b, p, pr)
    for a, k, pr in model.unimol:
        e.add_unimol_rxn(a, k, pr)
    if with_molecules:
        e.add_molecules(model.pos, model.species)
    return e


def engine_for(model: Model, precision="fp32", seed=1, capacity=0, with_molecules=True):
    """A prepared GPU engine holding the model (molecules optional)."""
    e = model_handle(model, precision, seed, capacity, with_molecules)
    e.prepare()
    return e
