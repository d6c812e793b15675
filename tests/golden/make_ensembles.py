#!/usr/bin/env python3
"""Ensemble fixtures: count trajectories of the oracle's serial engine (the reference's
scheduling semantics, oracle/mcell_oracle.c) for the ensemble-parity tests.

  ensemble_closed_cube.npz   the CPU-runnable configuration exactly: a reflective 1 um
                             cube, 5,000 A + 5,000 B uniform, A + B -> C at 1e8 /M/s
                             (P = 0.0368), dt = 1 us, 0.1 um subpartitions, 1,000
                             iterations; seeds 1..64 (initial positions and stream)
  ensemble_sphere_in_cube.npz  the large configuration reduced: an icosphere of
                             radius 0.5 um at 3 subdivision levels (1,280 triangles),
                             transparent to A, in a reflective 1.25 um cube; 60,000
                             molecules A:B 1:1, A + B -> C at 1e8 /M/s, C -> 0 at
                             1e3 /s, 200 iterations; seeds 1..48

Each file holds the counts of every species after every 10th iteration, per seed
(counts[seed, row, species], row k = iteration 10 (k + 1)). Seeded synthetic inputs
stand in for any dataset. Test infrastructure only.

Usage: python tests/golden/make_ensembles.py   (about a minute on 8 cores)
"""
from __future__ import annotations

import multiprocessing as mp
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

EVERY = 10
CONFIGS = {
    "closed_cube": dict(seeds=64, iterations=1000),
    "sphere_in_cube": dict(seeds=48, iterations=200),
}


def model(name, seed):
    from mcell_gb300 import workloads as W
    if name == "closed_cube":
        return W.closed_cube(n_per_species=5000, seed=seed)
    return W.sphere_in_cube(n_mol=60_000, seed=seed, levels=3, radius_um=0.5, cube_um=1.25, partition_um=1.35)


def run_one(job):
    name, seed, iters = job
    sys.path.insert(0, str(ROOT))
    from oracle.oracle_py import oracle_engine_for_model
    e = oracle_engine_for_model(model(name, seed), seed=seed)
    c = e.run(iters)
    return c[EVERY - 1::EVERY].astype(np.uint32)


def main():
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(8, mp.cpu_count())) as pool:
        for name, cfg in CONFIGS.items():
            t0 = time.time()
            jobs = [(name, s, cfg["iterations"]) for s in range(1, cfg["seeds"] + 1)]
            counts = np.stack(pool.map(run_one, jobs))
            np.savez_compressed(HERE / f"ensemble_{name}.npz", counts=counts, seeds=np.arange(1, cfg["seeds"] + 1),
                                every=EVERY, iterations=cfg["iterations"])
            print(f"{name}: {counts.shape} in {time.time() - t0:.0f} s; final mean {counts[:, -1].mean(0)}, "
                  f"sd {counts[:, -1].std(0, ddof=1)}")


if __name__ == "__main__":
    main()
