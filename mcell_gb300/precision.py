"""Precision form: the fp32 engine (fp32 positions and ray geometry, fp64
tie-breaks near planes and edges) measured against the fp64 engine, which
follows the reference routines bit for bit.

wall_hit_mismatch  the same diffusion cases (start molecule, injected
                   displacement and random draws) traced by both engines
                   through mcg_trace_cases; a case mismatches when the sequence
                   of wall events (kind and wall) differs. Two readings: each
                   engine starts from its own stored position (fp32 storage
                   rounds it, by up to half an ulp of the coordinate), or
                   (same_start) the fp64 engine holds the fp32 engine's stored
                   positions, so only the trace arithmetic differs
count_error        both engines run the model for n iterations with the same
                   seed; the species-count trajectories are compared, next to
                   two fp64 runs with different seeds (the stochastic scale)
"""
from __future__ import annotations

import numpy as np

from . import workloads as W

RESULT = 265  # doubles per traced case


def _wall_events(rows):
    out = []
    for r in rows:
        n = int(r[6])
        ev = r[9:9 + 8 * min(n, 32)].reshape(-1, 8)
        out.append(tuple((int(k), int(w)) for k, w in ev[:, :2] if k in (1, 2, 3)))
    return out


def fp32_stored(model: W.Model, e32=None) -> W.Model:
    """The model with each molecule at the position the fp32 engine stores for it
    (rounded to fp32 and, within a few ulp of a wall plane, moved off it on upload)."""
    from dataclasses import replace
    own = e32 is None
    e32 = e32 or W.engine_for(model, "fp32", seed=1)
    pos, sp, ids = e32.molecules()
    if own:
        e32.close()
    out = np.empty_like(model.pos)
    out[ids.astype(np.int64)] = pos
    return replace(model, pos=out)


def wall_hit_mismatch(model: W.Model, n_cases=100_000, near_ids=None, seed=5, chunk=20_000, e32=None, e64=None,
                      same_start=False):
    """Fraction of cases whose wall events differ between fp32 and fp64, and the
    largest final-position difference among the cases that agree (internal units).
    Half of the cases start from near_ids (e.g. molecules released next to edges)
    when given. Displacements are Gaussian with the species' space step.
    same_start: the fp64 engine starts from the fp32 engine's stored positions."""
    rng = np.random.default_rng(seed)
    n_mol = len(model.species)
    if near_ids is not None and len(near_ids):
        ids = np.concatenate([rng.choice(near_ids, n_cases // 2), rng.integers(0, n_mol, n_cases - n_cases // 2)])
    else:
        ids = rng.integers(0, n_mol, n_cases)
    sigma = model.space_steps[model.species[ids]] / np.sqrt(2.0)
    disp = rng.normal(size=(n_cases, 3)) * sigma[:, None]
    draws = rng.integers(0, 2 ** 32, size=(n_cases, 64), dtype=np.uint64).astype(np.uint32)
    own32, own64 = e32 is None, e64 is None
    e32 = e32 or W.engine_for(model, "fp32", seed=1)
    e64 = e64 or W.engine_for(fp32_stored(model, e32) if same_start else model, "fp64", seed=1)
    mism, err, hits = 0, 0.0, 0
    for a in range(0, n_cases, chunk):
        b = min(n_cases, a + chunk)
        r32 = e32.trace_cases(ids[a:b].astype(np.uint64), disp[a:b], draws[a:b])
        r64 = e64.trace_cases(ids[a:b].astype(np.uint64), disp[a:b], draws[a:b])
        w32, w64 = _wall_events(r32), _wall_events(r64)
        same = np.array([x == y for x, y in zip(w32, w64)])
        mism += int((~same).sum())
        hits += sum(1 for x in w64 if x)
        if same.any():
            err = max(err, float(np.abs(r32[same, 1:4] - r64[same, 1:4]).max()))
    if own32:
        e32.close()
    if own64:
        e64.close()
    return {"cases": n_cases, "cases_with_wall_events": hits, "mismatches": mism, "rate": mism / n_cases,
            "max_position_error": err, "same_start": bool(same_start)}


def count_error(model: W.Model, n_iter=50, seed=3):
    """Species-count trajectories of fp32 and fp64 runs (same seed) and of a second
    fp64 run (another seed): largest relative difference of the product count. Also
    the exact fallbacks each run took (mcg_get_fallbacks)."""
    traj, fallbacks = {}, {}
    for tag, prec, sd in (("fp32", "fp32", seed), ("fp64", "fp64", seed), ("fp64_other_seed", "fp64", seed + 1)):
        e = W.engine_for(model, prec, seed=sd)
        e.step(n_iter)
        traj[tag] = e.trajectory(n_iter).astype(np.float64)
        fallbacks[tag] = list(e.fallbacks())
        e.close()
    ref = np.maximum(traj["fp64"], 1.0)
    rel = np.abs(traj["fp32"] - traj["fp64"]) / ref
    noise = np.abs(traj["fp64_other_seed"] - traj["fp64"]) / ref
    return {"iterations": n_iter, "max_rel_error_fp32_vs_fp64": float(rel.max()),
            "max_rel_difference_two_fp64_seeds": float(noise.max()),
            "final_counts": {k: [int(x) for x in v[-1]] for k, v in traj.items()},
            "fallbacks_page_refills_walk_scans": fallbacks}
