"""Ensemble parity: species counts over time, the GPU engine against the oracle's
serial engine (the reference's scheduling: molecules in order, products and
reactions applied at once), mean and variance within 3 standard errors at every
10th iteration.

The GPU diffuses all molecules of an iteration at once against their partners'
start-of-iteration positions and resolves reactions by earliest claim; the serial
engine moves one molecule after another. These tests are the evidence that the
two schedules give the same count statistics. The oracle's trajectories are
committed fixtures (tests/golden/make_ensembles.py); the GPU runs the same models
(same builders, seeds 1..N) as replicas of one batch, each replica's result being
the same as the model run alone (tests/test_gpu_batch.py).
"""
import numpy as np
import pytest

from mcell_gb300 import _native
from mcell_gb300 import workloads as W
from tests import harness as H

pytestmark = pytest.mark.gpu


def _se_var(x):
    """Standard error of the sample variance along axis 0 (from the fourth central moment)."""
    n = x.shape[0]
    d = x - x.mean(0)
    m4 = (d ** 4).mean(0)
    v = x.var(0, ddof=1)
    return np.sqrt(np.maximum((m4 - (n - 3) / (n - 1) * v ** 2) / n, 0.0))


def compare_ensembles(g, o, label):
    """g, o: [runs, rows, species]. Returns the largest mean and variance z-scores."""
    g, o = g.astype(float), o.astype(float)
    ng, no = len(g), len(o)
    se_m = np.sqrt(g.var(0, ddof=1) / ng + o.var(0, ddof=1) / no)
    dm = np.abs(g.mean(0) - o.mean(0))
    z_m = np.where(se_m > 0, dm / np.where(se_m > 0, se_m, 1), np.where(dm > 0, np.inf, 0))
    se_v = np.sqrt(_se_var(g) ** 2 + _se_var(o) ** 2)
    dv = np.abs(g.var(0, ddof=1) - o.var(0, ddof=1))
    z_v = np.where(se_v > 0, dv / np.where(se_v > 0, se_v, 1), np.where(dv > 0, np.inf, 0))
    k = np.unravel_index(np.argmax(z_m), z_m.shape)
    print(f"{label}: max |z| of the mean {z_m.max():.2f} (row {k[0]}, species {k[1]}: gpu {g.mean(0)[k]:.1f}, "
          f"oracle {o.mean(0)[k]:.1f}), of the variance {z_v.max():.2f}; final means gpu {g.mean(0)[-1]} "
          f"oracle {o.mean(0)[-1]}")
    return z_m, z_v


def _gpu_ensemble(name, precision, builder):
    z = np.load(H.GOLDEN / f"ensemble_{name}.npz")
    seeds, iters, every = z["seeds"], int(z["iterations"]), int(z["every"])
    b = _native.Batch(precision, 3, len(seeds))
    hs = [W.model_handle(builder(int(s)), precision, seed=int(s)) for s in seeds]
    ids = b.add(hs)
    for h in hs:
        h.close()
    b.step(iters)
    g = np.stack([b.trajectory(r, iters)[every - 1::every] for r in ids])
    fb = b.fallbacks()
    b.close()
    return g, z["counts"], fb


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_closed_cube_ensemble_matches_oracle(precision):
    """The CPU-runnable configuration as stated: 10,000 molecules in a reflective 1 um
    cube, A + B -> C at P = 0.0368, 1,000 iterations, 64 seeds on each side."""
    g, o, fb = _gpu_ensemble("closed_cube", precision, lambda s: W.closed_cube(n_per_species=5000, seed=s))
    z_m, z_v = compare_ensembles(g, o, f"closed cube {precision}")
    assert (z_m <= 3).all() and (z_v <= 3).all()
    print("exact fallbacks taken:", fb)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sphere_in_cube_ensemble_matches_oracle(precision):
    """The large configuration reduced (icosphere of 1,280 triangles transparent to A in
    a reflective cube, 60,000 molecules, A + B -> C, C -> 0, 200 iterations, 48 seeds)."""
    g, o, fb = _gpu_ensemble("sphere_in_cube", precision, lambda s: W.sphere_in_cube(
        n_mol=60_000, seed=s, levels=3, radius_um=0.5, cube_um=1.25, partition_um=1.35))
    z_m, z_v = compare_ensembles(g, o, f"sphere in cube {precision}")
    assert (z_m <= 3).all() and (z_v <= 3).all()
    print("exact fallbacks taken:", fb)
