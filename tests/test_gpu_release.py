"""Volume releases generated on the device (ellipsoid, cuboid, shell, inside a
closed object): every molecule inside its region, uniform within it (moments within
5 standard errors), ids continuing the model's, and the model stepping on."""
import numpy as np
import pytest

from mcell_gb300 import conversion, geometry
from mcell_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _model():
    lu = conversion.length_unit_um()
    sv, sw = geometry.create_icosphere(0.6, 3)
    bv, bw = geometry.create_box(edge_dimension=1.6)
    v, w, obj = geometry.merge_meshes((sv, sw), (bv, bw))
    lay = conversion.partition_layout(v.min(0), v.max(0), partition_dimension_um=1.8, subpartition_dimension_um=0.1)
    steps, bimol, unimol = W._chemistry(1e-6, lu, conversion.default_rxn_radius_um())
    m = W.Model("release", lay.origin, lay.edge, lay.nsub, conversion.default_rxn_radius_um() / lu, v / lu, w,
                np.zeros((len(w), 3), np.uint8), steps, bimol, unimol, np.zeros((0, 3)), np.zeros(0, np.uint32))
    return m, obj


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_releases(precision):
    m, obj = _model()
    h = W.model_handle(m, precision, seed=3, capacity=400_000, with_molecules=False)
    h.set_wall_objects(obj)
    n = 60_000
    c = np.array([5.0, -3.0, 2.0])
    h.release(0, n, "sphere", c, (60.0, 40.0, 50.0), seed=11)
    h.release(1, n, "cuboid", c, (30.0, 20.0, 40.0), seed=12)
    h.release(0, n, "shell", (0, 0, 0), (50.0, 50.0, 50.0), seed=13)
    h.release(1, n, "inside", obj=0, seed=14)
    pos, sp, ids = h.molecules()
    assert len(ids) == 4 * n and np.array_equal(np.sort(ids), np.arange(4 * n))
    order = np.argsort(ids)
    pos, sp = pos[order], sp[order]
    sph, cub, shl, ins = pos[:n], pos[n:2 * n], pos[2 * n:3 * n], pos[3 * n:]
    # ellipsoid: inside, centred, <x^2> = a^2/5 per axis
    q = (sph - c) / np.array([30.0, 20.0, 25.0])
    assert ((q ** 2).sum(1) < 1 + 1e-6).all()
    assert np.abs(sph.mean(0) - c).max() < 5 * 30.0 / np.sqrt(5 * n)
    assert np.allclose((q ** 2).mean(0), 0.2, atol=5 * 0.18 / np.sqrt(n))
    # cuboid: inside, variance d^2 / 12
    d = np.array([30.0, 20.0, 40.0])
    assert (np.abs(cub - c) <= d / 2 + 1e-6).all()
    assert np.allclose(cub.var(0) / (d ** 2 / 12), 1.0, atol=0.03)
    # shell: on the sphere of radius 25
    assert np.allclose(np.linalg.norm(shl, axis=1), 25.0, rtol=1e-5)
    # inside the icosphere (inscribed in the 60-unit sphere): within it, and filling it
    r = np.linalg.norm(ins, axis=1)
    assert (r <= 60.0 + 1e-6).all()
    assert abs((r < 30.0).mean() - (30.0 / 58.5) ** 3) < 0.02  # polyhedron ~ a ball of radius ~58.5
    assert (sp[:n] == 0).all() and (sp[3 * n:] == 1).all()
    h.step(5)
    h.sync()
    h.close()


def test_model_without_molecules_steps_then_takes_a_release():
    # no molecules and no capacity reserved: the iterations run on empty arrays (counts
    # zero), as the reference's event does with an empty list; a release then fills it
    from mcell_gb300._native import Engine
    m, obj = _model()
    h = Engine("fp32", m.origin, m.partition_edge, m.nsub, m.rxn_radius, m.n_species, seed=5, capacity=0)
    h.set_species(m.space_steps)
    h.upload_mesh(m.verts, m.walls, m.wall_class)
    for a, b, p, pr in m.bimol:
        h.add_bimol_rxn(a, b, p, pr)
    for a, k, pr in m.unimol:
        h.add_unimol_rxn(a, k, pr)
    h.set_wall_objects(obj)
    h.prepare()
    h.step(3)
    assert (h.counts() == 0).all()
    assert (h.trajectory(3) == 0).all()
    h.release(0, 5000, "inside", obj=0, seed=21)
    h.step(4)
    c = h.counts()
    assert c[0] + c[2] == 5000 and c[1] == 0
    it, steps, _ = h.stats()
    assert it == 7 and steps >= 4 * 4000
    h.close()
