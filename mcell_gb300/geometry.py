"""Mesh builders for geometry objects (host side).

create_box follows the Model API's geometry_utils.create_box
(libmcell/api/geometry_utils.cpp:32-97): the same 8 vertices and 12 triangles in
the same order (CellBlender's), so wall indices match models built with the
reference API. create_icosphere subdivides an icosahedron by edge midpoints
projected back onto the sphere (the Model API's create_icosphere,
geometry_utils.cpp:228; there `subdivisions=1` is the bare icosahedron, here
`levels` counts the subdivision steps, so levels=5 gives 20,480 triangles).
create_bumpy_tube builds the precision-stress tube: a closed cylinder whose
radius is modulated by 0.05 um * sin of the axial and angular position.
All coordinates are in um; vertices are float64 [n, 3], walls uint32 [m, 3] with
outward normals (counter-clockwise seen from outside).
"""
from __future__ import annotations

import math
from typing import Tuple

import numpy as np


def create_box(edge_dimension: float = None, xyz_dimensions=None) -> Tuple[np.ndarray, np.ndarray]:
    if (edge_dimension is None) == (xyz_dimensions is None):
        raise ValueError("Exactly one edge_dimension or individual x, y, z dimensions can be set.")
    if edge_dimension is not None:
        x = y = z = edge_dimension / 2
    else:
        if len(xyz_dimensions) != 3:
            raise ValueError("Exactly one edge_dimension or individual x, y, z dimensions can be set.")
        x, y, z = (d / 2 for d in xyz_dimensions)
    verts = np.array([
        [-x, -y, -z], [-x, -y, z], [-x, y, -z], [-x, y, z],
        [x, -y, -z], [x, -y, z], [x, y, -z], [x, y, z]], dtype=np.float64)
    walls = np.array([
        [1, 2, 0], [3, 6, 2], [7, 4, 6], [5, 0, 4], [6, 0, 2], [3, 5, 7],
        [1, 3, 2], [3, 7, 6], [7, 5, 4], [5, 1, 0], [6, 4, 0], [3, 1, 5]], dtype=np.uint32)
    return verts, walls


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([
        [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
        [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
        [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    return v, np.array(f, dtype=np.int64)


def create_icosphere(radius: float, levels: int, center=(0.0, 0.0, 0.0)) -> Tuple[np.ndarray, np.ndarray]:
    if levels < 0 or levels > 7:
        raise ValueError("levels must be in 0..7")
    verts, faces = _icosahedron()
    for _ in range(levels):
        vlist = list(verts)
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                m /= np.linalg.norm(m)
                cache[key] = len(vlist)
                vlist.append(m)
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        verts = np.array(vlist)
        faces = np.array(nf, dtype=np.int64)
    verts = verts * radius + np.asarray(center, dtype=np.float64)
    return verts.astype(np.float64), faces.astype(np.uint32)


def create_star_sphere(radius: float, levels: int, bump: float = 0.35, center=(0.0, 0.0, 0.0)):
    """A closed, non-convex mesh: an icosphere whose vertices sit at radius
    r(theta, phi) = radius * (1 + bump * sin(3 phi) * sin(2 theta)) (deep lobes and
    dents; outward-facing normals as the icosphere's)."""
    v, w = create_icosphere(1.0, levels)
    th = np.arccos(np.clip(v[:, 2], -1.0, 1.0))
    ph = np.arctan2(v[:, 1], v[:, 0])
    r = radius * (1.0 + bump * np.sin(3.0 * ph) * np.sin(2.0 * th))
    return (v * r[:, None] + np.asarray(center, dtype=np.float64)).astype(np.float64), w


def create_bumpy_tube(radius: float = 0.2, length: float = 10.0, bump: float = 0.05,
                      n_theta: int = 200, n_z: int = 500, axial_waves: float = 20.0,
                      angular_waves: int = 4) -> Tuple[np.ndarray, np.ndarray]:
    """Closed tube along z centred at the origin, r = radius + bump*sin(2pi*w*z/L)*sin(k*theta).

    Triangles: 2 * n_theta * n_z on the side plus 2 * n_theta on the end caps
    (n_theta=200, n_z=500 gives 200,400)."""
    th = np.arange(n_theta) * (2 * math.pi / n_theta)
    zs = np.linspace(-length / 2, length / 2, n_z + 1)
    verts = []
    for z in zs:
        r = radius + bump * np.sin(2 * math.pi * axial_waves * (z + length / 2) / length) * np.sin(angular_waves * th)
        verts.append(np.stack([r * np.cos(th), r * np.sin(th), np.full_like(th, z)], axis=1))
    verts = np.concatenate(verts)
    faces = []
    for j in range(n_z):
        for i in range(n_theta):
            a = j * n_theta + i
            b = j * n_theta + (i + 1) % n_theta
            c = (j + 1) * n_theta + (i + 1) % n_theta
            d = (j + 1) * n_theta + i
            faces += [[a, b, c], [a, c, d]]
    c0 = len(verts)
    c1 = c0 + 1
    verts = np.concatenate([verts, [[0, 0, -length / 2], [0, 0, length / 2]]])
    top = n_z * n_theta
    for i in range(n_theta):
        faces.append([c0, (i + 1) % n_theta, i])
        faces.append([c1, top + i, top + (i + 1) % n_theta])
    return verts.astype(np.float64), np.array(faces, dtype=np.uint32)


def merge_meshes(*meshes):
    """Concatenate (verts, walls) meshes into one vertex/wall list and object ids per wall."""
    vs, ws, obj = [], [], []
    off = 0
    for k, (v, w) in enumerate(meshes):
        vs.append(v)
        ws.append(w.astype(np.int64) + off)
        obj.append(np.full(len(w), k, dtype=np.uint32))
        off += len(v)
    return np.concatenate(vs), np.concatenate(ws).astype(np.uint32), np.concatenate(obj)
