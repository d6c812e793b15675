"""Checkpoints and visualisation files from device state.

A run restored from a checkpoint must repeat the uninterrupted run: the same count
trajectory and, at the end, the same molecules (ids, species, positions bit for bit),
since the random streams are counter based (seed, molecule id, iteration). Viz files
must hold exactly the downloaded molecules in the reference's formats."""
import struct

import numpy as np
import pytest

from mcell_gb300 import checkpoint
from mcell_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NAMES = ["A", "B", "C"]


def _by_id(pos, sp, ids):
    o = np.argsort(ids)
    return pos[o], sp[o], ids[o]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_checkpoint_continues_the_run(tmp_path, precision):
    m = W.replica_models(1, seed=41, n_range=(6_000, 6_001), edge_range_um=(0.8, 0.8), k_range=(1e8, 1e8),
                         sphere_fraction=1.0, levels=(3, 3))[0]
    full = W.engine_for(m, precision, seed=9)
    full.step(40)
    want = full.trajectory(40)
    wp, ws, wi = _by_id(*full.molecules())
    first = W.engine_for(m, precision, seed=9)
    first.step(20)
    st = checkpoint.save(first, tmp_path / "ck.npz")
    assert st["iteration"] == 20 and (st["flags"] <= 1).all()
    assert (st["unimol_time"] < 1e19).any() or want[-1, 2] == 0  # products carry drawn unimolecular times
    second = W.model_handle(m, precision, seed=9, with_molecules=False)
    checkpoint.load(second, tmp_path / "ck.npz")
    assert np.array_equal(second.counts(), want[19])
    second.step(20)
    assert np.array_equal(second.trajectory(20), want[20:])
    gp, gs, gi = _by_id(*second.molecules())
    assert np.array_equal(gi, wi) and np.array_equal(gs, ws) and np.array_equal(gp, wp)


def test_viz_files_hold_the_molecules(tmp_path):
    m = W.closed_cube(n_per_species=1000, seed=3)
    e = W.engine_for(m, "fp32", seed=2)
    e.step(5)
    pos, sp, ids = e.molecules()
    prefix = tmp_path / "viz_data" / "seed_00001" / "Scene"
    e.write_viz(prefix, NAMES, 5, 1000, mode="ascii")
    rows = (tmp_path / "viz_data" / "seed_00001" / "Scene.ascii.0005.dat").read_text().split("\n")[:-1]
    assert len(rows) == len(ids)
    got = {int(r.split()[1]): (r.split()[0], np.array([float(x) for x in r.split()[2:5]])) for r in rows}
    for k in range(0, len(ids), 97):
        name, xyz = got[int(ids[k])]
        assert name == NAMES[sp[k]] and np.allclose(xyz, pos[k] * 0.01, rtol=1e-8, atol=0)
    e.write_viz(prefix, NAMES, 5, 1000, mode="cellblender_v2")
    b = (tmp_path / "viz_data" / "seed_00001" / "Scene.cellbin.0005.dat").read_bytes()
    assert struct.unpack_from("<I", b, 0)[0] == 2
    off, seen = 4, 0
    while off < len(b):
        (ln,) = struct.unpack_from("<I", b, off)
        name = b[off + 4:off + 4 + ln].decode()
        off += 4 + ln
        assert b[off] == 0
        (cnt,) = struct.unpack_from("<I", b, off + 1)
        off += 5
        fid = np.frombuffer(b, np.uint32, cnt, off)
        off += 4 * cnt
        xyz = np.frombuffer(b, np.float32, 3 * cnt, off).reshape(cnt, 3)
        off += 12 * cnt
        a = NAMES.index(name)
        sel = sp == a
        assert sorted(fid.tolist()) == sorted(ids[sel].astype(np.uint32).tolist())
        assert np.allclose(np.sort(xyz[:, 0]), np.sort((pos[sel, 0] * 0.01).astype(np.float32)))
        seen += cnt
    assert seen == len(ids)


def test_count_files_in_the_reference_formats(tmp_path):
    """DAT ("time value" per line, C++ stream defaults) and GDAT (a '#' header of
    right-aligned names, then scientific numbers with two-digit exponents) written from
    the device counts: the same numbers as the count trajectory, in the world and
    inside a counted object."""
    from tests.test_gpu_counted import _model as counted_model

    m, obj, _, _ = counted_model()
    h = W.model_handle(m, "fp32", seed=4)
    h.set_wall_objects(obj)
    h.set_counted_objects([0])
    h.prepare()
    world0 = h.counts()
    inside0 = h.counted_counts()
    h.step(12)
    world = h.trajectory(12)
    inside = h.counted_trajectory(12)
    cols = [(0, -1, "A_world"), (2, -1, "C_world"), (0, 0, "A_in_sphere")]
    h.write_counts(tmp_path / "run", cols, n_iterations=12, every=3, time_step_s=1e-6, fmt="dat")
    h.write_counts(tmp_path / "run", cols, n_iterations=12, every=3, time_step_s=1e-6, fmt="gdat")
    h.close()
    # the window reaches back to the start: a t = 0 row of the counts before the first
    # iteration (the reference's count event runs before diffusion in iteration 0),
    # then iterations 3, 6, 9, 12
    rows = [2, 5, 8, 11]
    times = [0.0, 3e-6, 6e-6, 9e-6, 1.2e-5]
    want = {"A_world": np.r_[world0[0], world[rows, 0]], "C_world": np.r_[world0[2], world[rows, 2]],
            "A_in_sphere": np.r_[inside0[0, 0], inside[rows, 0, 0]]}
    for name, vals in want.items():
        lines = (tmp_path / f"run.{name}.dat").read_text().splitlines()
        assert lines[0].split()[0] == "0" and lines[1].split()[0] == "3e-06" and lines[4].split()[0] == "1.2e-05"
        got = np.array([[float(x) for x in ln.split()] for ln in lines])
        assert np.allclose(got[:, 0], times) and np.array_equal(got[:, 1], vals.astype(float))
    text = (tmp_path / "run.gdat").read_text().splitlines()
    assert text[0] == "#" + "time".rjust(14) + "".join(n.rjust(16) for n in ("A_world", "C_world", "A_in_sphere"))
    first = text[1].split()
    assert text[1].startswith(" 0.00000000e+00  ") and len(first) == 4
    assert text[2].startswith(" 3.00000000e-06  ")
    g = np.array([[float(x) for x in ln.split()] for ln in text[1:]])
    for k, name in enumerate(("A_world", "C_world", "A_in_sphere")):
        assert np.array_equal(g[:, k + 1], want[name].astype(float))
