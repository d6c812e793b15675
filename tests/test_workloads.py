"""The synthetic models start with every molecule inside their closed meshes (no GPU).

A molecule released outside a closed mesh diffuses freely until it leaves the
partition, which the engine reports as MCG_ERR_ESCAPE (the reference's fatal error).
The bumpy tube's near-edge molecules are the delicate case: they sit within 1 nm of a
mesh edge or vertex. Membership is decided exactly on the tube's own facets: the
side mesh is a grid of rings (angle i, height j), so the ray from the axis at a point's
height and angle crosses the side in the one quad of that (angle, height) cell, and
the point is inside when it is nearer the axis than that crossing."""
import numpy as np
import pytest

from mcell_gb300 import workloads as W

N_THETA = 200


def _outside(verts, pos, n_theta, n_z):
    """Indices of points outside the tube side (or beyond its end caps)."""
    z0, z1 = verts[0, 2], verts[n_z * n_theta, 2]
    dz = (z1 - z0) / n_z
    th = np.mod(np.arctan2(pos[:, 1], pos[:, 0]), 2 * np.pi)
    i = np.minimum((th / (2 * np.pi / n_theta)).astype(np.int64), n_theta - 1)
    j = np.clip(np.floor((pos[:, 2] - z0) / dz).astype(np.int64), 0, n_z - 1)
    a = verts[j * n_theta + i]
    b = verts[j * n_theta + (i + 1) % n_theta]
    c = verts[(j + 1) * n_theta + (i + 1) % n_theta]
    d = verts[(j + 1) * n_theta + i]
    o = np.stack([np.zeros(len(pos)), np.zeros(len(pos)), pos[:, 2]], axis=1)
    u = np.stack([np.cos(th), np.sin(th), np.zeros(len(pos))], axis=1)

    def hit(p0, p1, p2):
        # Moller-Trumbore: distance along u and the barycentric coordinates
        e1, e2 = p1 - p0, p2 - p0
        h = np.cross(u, e2)
        det = (e1 * h).sum(1)
        s = o - p0
        bu = (s * h).sum(1) / det
        q = np.cross(s, e1)
        bv = (u * q).sum(1) / det
        t = (e2 * q).sum(1) / det
        ok = (bu >= -1e-9) & (bv >= -1e-9) & (bu + bv <= 1 + 1e-9)
        return np.where(ok, t, np.nan)

    t = hit(a, b, c)
    t = np.where(np.isnan(t), hit(a, c, d), t)
    assert not np.isnan(t).any()
    r = np.hypot(pos[:, 0], pos[:, 1])
    out = (r >= t) | (pos[:, 2] <= z0) | (pos[:, 2] >= z1)
    return np.nonzero(out)[0]


@pytest.mark.parametrize("kw", [dict(n_mol=200_000, length_um=2.0, n_z=100, subparts_per_edge=100),
                                dict(n_mol=1_000_000, seed=2), dict(n_mol=400_000)])
def test_bumpy_tube_molecules_start_inside(kw):
    m = W.bumpy_tube(**kw)
    n_z = kw.get("n_z", 500)
    bad = _outside(m.verts, m.pos, N_THETA, n_z)
    assert len(bad) == 0, (len(bad), m.pos[bad[:3]])


def test_the_inside_check_sees_a_molecule_outside():
    # a near-edge molecule an earlier placement put just outside the side, 0.2 units
    # below the cap (where the clip to the cap had moved it)
    m = W.bumpy_tube(n_mol=1000)
    p = np.array([[18.903875350952, 6.315864086151, 499.799987792969], [18.0, 6.0, 499.0], [0.0, 0.0, 0.0]])
    assert _outside(m.verts, p, N_THETA, 500).tolist() == [0]
