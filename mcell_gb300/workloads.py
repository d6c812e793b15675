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
