#!/usr/bin/env python3
"""Benchmark of the volume-molecule diffuse-react step on one GB300.

Workload (one step = one iteration of the whole model): an icosphere of radius
1 um with 20,480 triangles, transparent to A and reflective to B and C, centred
in a reflective 2.5 um cube (20,492 walls); 1,000,000 molecules, A:B 1:1
uniform in the cube; D = 1e-6 cm^2/s (C: 5e-7); A + B -> C at 1e8 M^-1 s^-1;
C -> 0 at 1e3 s^-1; dt = 1 us; fp32 positions; subpartitions of 0.1 um.
Synthetic, seeded inputs (no dataset exists for this configuration).

Metric: molecule-steps/s = live volume molecules at the start of each step,
summed over the timed steps, over the device time of those steps.
  value  device time (CUDA events on the engine's stream) per step, with the L2
         flushed (a 512 MB write) before every timed step
  e2e    the same metric through the C ABI with host buffers: the molecule
         upload from host memory and, every step, mcg_step + a device-to-host
         read of the species counts (mcg_request_counts after the step, waited
         for once the next step is queued), timed on the host
Arms:
  default            the CUDA engine (mcell_gb300)
  --impl reference   the reference algorithm on the host cores: the oracle's
                     serial engine (a restatement of MCell4's step; the
                     reference itself cannot be built), one seeded process per
                     core as MCell4 is single-threaded
Multi-GPU: replicas only (independent models per rank, no collectives).
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "molecule-steps/s @1M mols,20k tris; batched/served vs plain GPU; p50/p99 latency"
UNIT = "molecule-steps/s"
ALG_BYTES_PER_MOL_STEP = 32  # read a 16 B record + write a 16 B record


def _rank_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ---------------------------------------------------------------- CPU (oracle) leg

def _cpu_worker(args):
    n_mol, iters, seed = args
    from mcell_gb300 import workloads
    from oracle.oracle_py import oracle_engine_for_model

    m = workloads.sphere_in_cube(n_mol=n_mol, seed=seed)
    e = oracle_engine_for_model(m, seed=seed)
    t0 = time.perf_counter()
    e.run(iters)
    dt = time.perf_counter() - t0
    steps = e.lib.orc_engine_mol_steps(e.h)
    return steps, dt


def cpu_measure(procs, n_mol, iters, pool=None):
    """Aggregate mol-steps/s of `procs` independent seeded processes (spawned)."""
    args = [(n_mol, iters, 1000 + k) for k in range(procs)]
    if pool is None:
        with mp.get_context("spawn").Pool(procs) as p:
            res = p.map(_cpu_worker, args)
    else:
        res = pool.map(_cpu_worker, args)
    rate = sum(s / dt for s, dt in res)
    return rate, res


def _ensure_oracle_built():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)


# ---------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.idx = gpu_index
        self.p = None

    def _lines(self):
        self.f.flush()
        try:
            with open(self.f.name) as fh:
                return sum(1 for _ in fh)
        except OSError:
            return 0

    def __enter__(self):
        # sampling every 20 ms; the timed region starts once nvidia-smi has written its
        # first row (it takes ~0.1 s to start), and rows from before it are dropped
        self.skip = 0
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        if self.p:
            t0 = time.time()
            while self._lines() == 0 and time.time() - t0 < 5 and self.p.poll() is None:
                time.sleep(0.01)
            self.skip = self._lines()
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if len(rows) > self.skip:
            rows = rows[self.skip:]  # the timed region's rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- GPU leg

def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_per_mol_step():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("k_diffuse_dram_bytes_per_mol_step")
    return None


def combine_ranks(seconds, units, world, device):
    """Whole-job figures of a replicas-only run: the slowest rank's time (max) and the
    units every rank processed (sum). One rank: the inputs. `device` is where the
    reduction tensors live ("cuda" under NCCL, "cpu" under gloo)."""
    if world <= 1:
        return float(seconds), float(units)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    n = torch.tensor([float(units)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(n, op=torch.distributed.ReduceOp.SUM)
    return t.item(), n.item()


def workload_name(n_mol):
    """The main line's workload, named by what it is (1M molecules unless --n-mol says otherwise)."""
    count = "1M" if n_mol == 1_000_000 else f"{n_mol:,}"
    return ("sphere_in_cube: icosphere r=1um 20480 tris transparent to A in a 2.5um reflective cube, "
            f"{count} molecules A:B 1:1, A+B->C 1e8/M/s, C->0 1e3/s, dt=1us")


def run_gpu(args, rank, world):
    import numpy as np
    import torch

    from mcell_gb300 import workloads

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    # replicas: every rank simulates its own seeded model
    model = workloads.sphere_in_cube(n_mol=args.n_mol, seed=1 + rank)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    e = workloads.engine_for(model, "fp32", seed=7 + rank)
    e.set_options(use_graphs=True, profile=True)
    for _ in range(args.warmup):
        e.step(1)
    e.sync()
    e.profile()
    _, ms0, l0 = e.stats()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    prof = np.zeros(6)
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (on torch's stream, finished before the step)
            torch.cuda.synchronize()
            e.step(1)
            e.sync()
            prof += e.profile()
    torch.cuda.synchronize()
    _, ms1, l1 = e.stats()
    fallbacks = e.fallbacks()
    clocks = clk.summary()
    mol_steps = ms1 - ms0
    iter_ms = prof[0]
    t_ms, all_steps = combine_ranks(iter_ms, mol_steps, world, "cuda")
    value = all_steps / (t_ms / 1e3)
    diffuse_ms_per_launch = prof[1] / args.steps
    mols_per_launch = mol_steps / args.steps
    achieved = ALG_BYTES_PER_MOL_STEP * mols_per_launch / (diffuse_ms_per_launch / 1e3) / 1e9
    peak, peak_kind = _peaks()
    tpm = _traffic_per_mol_step()
    # graph-replay throughput without flushes (steady state, informative)
    e.set_options(use_graphs=True, profile=False)
    e.sync()
    _, a0, _ = e.stats()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.step(args.steps if args.steps % 2 == 0 else args.steps + 1)
    e.sync()
    graph_s = time.perf_counter() - t0
    _, a1, _ = e.stats()
    graph_rate = (a1 - a0) / graph_s
    e.close()

    # end to end through the C ABI, host buffers in and out
    e2 = workloads.engine_for(model, "fp32", seed=7 + rank, with_molecules=False)
    pos = np.ascontiguousarray(model.pos, np.float64)
    sp = np.ascontiguousarray(model.species, np.uint32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2.add_molecules(pos, sp)
    # every step's counts are read, one step late: the copy is queued behind the step
    # and waited for while the device runs the next one
    counts, prev = None, None
    for _ in range(args.steps):
        e2.step(1)
        t = e2.request_counts()
        if prev is not None:
            counts = e2.wait_counts(prev)
        prev = t
    counts = e2.wait_counts(prev)
    e2_s = time.perf_counter() - t0
    _, e2_steps, _ = e2.stats()
    e2.close()
    e2e_s_all, e2e_steps_all = combine_ranks(e2_s, e2_steps, world, "cuda")
    h2d = pos.nbytes + sp.nbytes
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform release; icosphere + cube mesh generated)",
        "config": {"workload": workload_name(args.n_mol),
                   "molecules": args.n_mol, "walls": int(len(model.walls)), "subparts_per_edge": int(model.nsub),
                   "precision": "fp32 positions", "parallelism": f"replicas x{world}",
                   "l2": "flushed (512 MB write) before every timed step"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "kernel": "k_diffuse",
                     "algorithmic_bytes_per_mol_step": ALG_BYTES_PER_MOL_STEP,
                     "traffic": (tpm * mols_per_launch) if tpm else None},
        # read back per step: the species counts and the 64-byte head of the engine's
        # counters (status word and iteration) that mcg_wait_counts checks
        "e2e": {"value": e2e_steps_all / e2e_s_all, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": 8 * model.n_species + 64},
        "gpu_launches": int(l1 - l0),
        "clocks": clocks,
        "kernel_ms_per_step": {"diffuse": prof[1] / args.steps, "reactions": prof[2] / args.steps,
                               "products": prof[3] / args.steps, "sort": prof[4] / args.steps},
        "graph_replay_value": graph_rate,
        "final_counts": [int(x) for x in counts] if counts is not None else None,
        "fallbacks": {"page_refills": fallbacks[0], "walk_scans": fallbacks[1],
                      "note": "ray traces since upload that took the exact fallbacks of the fixed-size candidate "
                              "page (16) and partner list (48); results do not depend on them"},
    }
    return line


# ---------------------------------------------------------------- batching form

def run_batching(args):
    """Independent replicas (the batching distribution of workloads.replica_models)
    for args.batch_iters iterations: all in one batch (one launch per kernel per
    iteration, CUDA graphs, autotuned) against the same models run one after
    another on the plain engine (graphs on). Both fp32. Times are host wall
    clock around step + sync of the whole job; model upload is reported apart."""
    import torch

    from mcell_gb300 import _native
    from mcell_gb300 import workloads as W

    models = W.replica_models(args.batch_replicas, seed=7)
    iters = args.batch_iters
    n_mol = sum(len(m.species) for m in models)
    # batched
    t0 = time.perf_counter()
    b = _native.Batch("fp32", 3, len(models), autotune=True)
    hs = [W.model_handle(m, "fp32", seed=1000 + k) for k, m in enumerate(models)]
    ids = b.add(hs)
    for h in hs:
        h.close()
    b.sync()
    setup_b = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.step(iters)
    b.sync()
    job_b = time.perf_counter() - t0
    _, steps_b, launches_b = b.stats()
    fallbacks_b = b.fallbacks()
    finals_b = [b.counts(r) for r in ids]
    blocks = b.diffuse_blocks_per_sm()
    mem_b = b.device_bytes()
    b.close()
    # plain engine, one model after another
    job_p, setup_p, steps_p = 0.0, 0.0, 0
    for k, m in enumerate(models):
        t0 = time.perf_counter()
        e = W.engine_for(m, "fp32", seed=1000 + k)
        e.sync()
        t1 = time.perf_counter()
        e.step(iters)
        e.sync()
        t2 = time.perf_counter()
        _, st, _ = e.stats()
        steps_p += st
        setup_p += t1 - t0
        job_p += t2 - t1
        e.close()
    return {
        "workload": f"{len(models)} replicas: cubes 0.5-3 um (log-uniform), half with an icosphere (level 2-5, "
                    f"r = 0.4 edge, transparent to A), 1k-200k molecules (log-uniform, {n_mol} in total), "
                    f"A+B->C k 1e6-1e9 /M/s (log-uniform), C->0 1e3/s, dt 1 us, fp32, {iters} iterations",
        "batched": {"job_s": job_b, "setup_s": setup_b, "replicas_per_hour": 3600.0 * len(models) / job_b,
                    "molecule_steps_per_s": steps_b / job_b, "diffuse_blocks_per_sm": blocks,
                    "device_bytes": mem_b, "launches": launches_b},
        "plain_sequential": {"job_s": job_p, "setup_s": setup_p, "replicas_per_hour": 3600.0 * len(models) / job_p,
                             "molecule_steps_per_s": steps_p / job_p},
        "speedup_replicas_per_hour": job_p / job_b,
        "final_counts_replica0": [int(x) for x in finals_b[0]],
        "fallbacks_batched": {"page_refills": fallbacks_b[0], "walk_scans": fallbacks_b[1]},
        "note": f"both arms run {iters} iterations of each replica; replicas_per_hour is for jobs of that length",
    }


# ---------------------------------------------------------------- closed cube (CPU-runnable case)

def _cube_cpu_worker(args):
    seed, iters = args
    from mcell_gb300 import workloads
    from oracle.oracle_py import oracle_engine_for_model

    m = workloads.closed_cube(seed=seed)
    e = oracle_engine_for_model(m, seed=seed)
    t0 = time.perf_counter()
    e.run(iters)
    dt = time.perf_counter() - t0
    return e.lib.orc_engine_mol_steps(e.h), dt


def run_closed_cube(args, cpu_pool=None):
    """The reference's CPU-runnable configuration: a reflective 1 um cube, A and B
    5,000 each, A+B->C, fp64, 1,000 iterations, seeds 1..8 — each seed run alone on
    the plain engine, all eight as one batch, and (when a pool of host processes is
    given) the oracle's serial engine for 100 iterations per seed, one process per
    seed."""
    from mcell_gb300 import _native
    from mcell_gb300 import workloads as W

    seeds = list(range(1, 9))
    iters = 1000
    models = [W.closed_cube(seed=sd) for sd in seeds]
    alone_s, steps_alone = 0.0, 0
    for sd, m in zip(seeds, models):
        e = W.engine_for(m, "fp64", seed=sd)
        e.sync()
        t0 = time.perf_counter()
        e.step(iters)
        e.sync()
        alone_s += time.perf_counter() - t0
        steps_alone += e.stats()[1]
        e.close()
    b = _native.Batch("fp64", 3, len(models))
    hs = [W.model_handle(m, "fp64", seed=sd) for sd, m in zip(seeds, models)]
    b.add(hs)
    for h in hs:
        h.close()
    b.sync()
    t0 = time.perf_counter()
    b.step(iters)
    b.sync()
    batch_s = time.perf_counter() - t0
    steps_batch = b.stats()[1]
    b.close()
    out = {"workload": "closed 1 um cube, 12 reflective walls, A 5,000 + B 5,000, A+B->C 1e8/M/s, dt 1 us, "
                       "fp64, 1,000 iterations, seeds 1..8",
           "plain_gpu_one_seed_after_another": {"job_s": alone_s, "molecule_steps_per_s": steps_alone / alone_s},
           "batched_gpu_8_seeds": {"job_s": batch_s, "molecule_steps_per_s": steps_batch / batch_s}}
    if cpu_pool is not None:
        res = cpu_pool.map(_cube_cpu_worker, [(sd, 100) for sd in seeds])
        out["cpu_oracle_8_processes"] = {"molecule_steps_per_s": sum(st / dt for st, dt in res), "cores": len(seeds),
                                         "sample": "100 of the 1,000 iterations per seed"}
    return out


# ---------------------------------------------------------------- precision form

def run_precision(args):
    """fp32 engine (fp64 tie-breaks) against the fp64 engine on the bumpy tube:
    wall-hit identity on 100,000 traced cases of the full model (10M molecules,
    200,400 triangles; half of the cases start within 1 nm of an edge or vertex),
    once with each engine at its own stored positions and once with the fp64 engine
    at the fp32 engine's (trace arithmetic alone), and the count trajectories of a tube
    of args.precision_count_molecules molecules over args.precision_iters iterations
    (by default the model as configured, 10M x 500: about a minute for the three runs,
    the fp64 ones slowest while most molecules are still unreacted)."""
    import numpy as np

    from mcell_gb300 import precision
    from mcell_gb300 import workloads as W

    m = W.bumpy_tube(n_mol=10_000_000)
    n = len(m.species)
    near = np.arange(n - int(round(0.05 * n)), n)
    mism = precision.wall_hit_mismatch(m, n_cases=100_000, near_ids=near)
    mism_same = precision.wall_hit_mismatch(m, n_cases=100_000, near_ids=near, same_start=True)
    nc = args.precision_count_molecules
    if nc != n:
        del m
        m = W.bumpy_tube(n_mol=nc, seed=2)
    cnt = precision.count_error(m, n_iter=args.precision_iters)
    out = {"workload": "bumpy tube r = 0.2 um (+-0.05 um), 10 um, 200,400 reflective triangles, 5% of the molecules "
                       "within 1 nm of edges/vertices, A+B->C, dt 0.1 us",
           "wall_hit_mismatch_10M": mism, "wall_hit_mismatch_10M_same_start": mism_same,
           f"count_error_{nc // 1_000_000}M_{args.precision_iters}_iterations": cnt}
    if (nc, args.precision_iters) != (n, 500):
        out["reduction"] = f"count error on a {nc:,}-molecule tube over {args.precision_iters} iterations, not 10M x 500"
    return out


# ---------------------------------------------------------------- serving form

def run_serving(rate, seconds, plain=True, seed=11):
    """Requests drawn from the batching distribution with iteration counts
    log-uniform in 100-10,000 arrive as a Poisson stream (rate per s for `seconds`)
    and are served by the continuous-batching loop (mcg_serve_*; slots 256,
    device-memory budget 150 GB). Time-to-result is measured per request from
    submission to result. With `plain`, the same requests are then run one after
    another on the plain engine; their time-to-result under first-come,
    first-served is computed from those measured run times and the same arrivals.
    Without it, the offered load is set against the plain engine's capacity (the
    molecule-steps/s it sustains on this distribution, `plain_capacity`)."""
    import numpy as np

    from mcell_gb300 import _native
    from mcell_gb300 import workloads as W

    rng = np.random.default_rng(seed)
    n_req = max(1, int(rng.poisson(rate * seconds)))
    arrivals = np.sort(rng.uniform(0, seconds, n_req))
    iters = np.exp(rng.uniform(np.log(100), np.log(10_000), n_req)).astype(int)
    models = W.replica_models(n_req, seed=seed)
    offered = float(sum(len(m.species) * int(k) for m, k in zip(models, iters))) / seconds
    handles = [W.model_handle(m, "fp32", seed=2000 + k) for k, m in enumerate(models)]
    srv = _native.Server("fp32", 3, max_slots=256, hbm_budget_bytes=150 << 30, autotune=True)
    t0 = time.perf_counter()
    tickets = []
    for k in range(n_req):
        delay = arrivals[k] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        tickets.append(srv.submit(handles[k], int(iters[k])))
    lat = []
    for t in tickets:
        assert srv.wait(t, 3600.0) == "done"
        lat.append(srv.poll(t)[1])
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    mol_steps = float(st["mol_steps"])
    out = {
        "workload": f"{n_req} requests, Poisson {rate}/s over {seconds} s, models of the batching distribution, "
                    f"iterations log-uniform 100-10000 ({int(iters.sum())} in total), fp32",
        "offered_molecule_steps_per_s": offered,
        "served": {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                   "makespan_s": wall, "molecule_steps_per_s": mol_steps / wall,
                   "busy_molecule_steps_per_s": mol_steps / max(st["busy_seconds"], 1e-9)},
    }
    if plain:
        # plain engine, one request after another (first come, first served)
        service = []
        for k, m in enumerate(models):
            e = W.engine_for(m, "fp32", seed=2000 + k)
            e.sync()
            t1 = time.perf_counter()
            e.step(int(iters[k]))
            e.sync()
            service.append(time.perf_counter() - t1)
            e.close()
        done, plain_lat = 0.0, []
        for a, sv in zip(arrivals, service):
            done = max(done, a) + sv
            plain_lat.append(done - a)
        out["plain_sequential"] = {"p50_s": float(np.percentile(plain_lat, 50)),
                                   "p99_s": float(np.percentile(plain_lat, 99)), "makespan_s": float(done),
                                   "molecule_steps_per_s": mol_steps / max(sum(service), 1e-9)}
    for h in handles:
        h.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-mol", type=int, default=1_000_000)
    ap.add_argument("--cpu-procs", type=int, default=0, help="CPU processes (0 = all host cores)")
    ap.add_argument("--cpu-iters", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batching measurement")
    ap.add_argument("--batch-replicas", type=int, default=256)
    ap.add_argument("--batch-iters", type=int, default=1000)
    ap.add_argument("--no-cube", action="store_true", help="skip the closed-cube measurement")
    ap.add_argument("--no-precision", action="store_true", help="skip the precision measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="the overload burst's arrival rate")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="the overload burst's duration")
    ap.add_argument("--sustained-rate", type=float, default=10.0)
    ap.add_argument("--sustained-seconds", type=float, default=60.0, help="0 skips the sustained serving run")
    ap.add_argument("--precision-iters", type=int, default=500)
    ap.add_argument("--precision-count-molecules", type=int, default=10_000_000,
                    help="molecules of the tube whose count trajectories are compared (10M: the model as configured)")
    args = ap.parse_args()
    rank, world, _ = _rank_env()
    procs = args.cpu_procs or os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return 0
        _ensure_oracle_built()
        # each step: one iteration of the full model on every host core (independent seeds)
        with mp.get_context("spawn").Pool(procs) as pool:
            rate_w, _ = cpu_measure(procs, args.n_mol, 1, pool)  # warm-up pass (setup + first iteration)
            t_all, steps_all = 0.0, 0
            for _ in range(max(1, min(args.steps, 3))):
                r, res = cpu_measure(procs, args.n_mol, args.cpu_iters, pool)
                steps_all += sum(s for s, _ in res)
                t_all += max(dt for _, dt in res)
        value = steps_all / t_all
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": workload_name(args.n_mol), "molecules": args.n_mol,
                           "precision": "fp64 positions (the oracle's serial engine restates the reference's fp64 "
                                        "build; the GPU arm computes positions in fp32)",
                           "parallelism": f"{procs} independent seeded processes (MCell4 is single-threaded)"},
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                                 "sample": f"{procs} processes x {args.cpu_iters} iterations of the {args.n_mol:,}-molecule model "
                                           f"per step, up to 3 steps"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    # our arm: CPU baseline first (spawned processes, before any GPU call)
    cpu = None
    cube_pool = None
    if rank == 0 and not args.no_cpu_baseline:
        _ensure_oracle_built()
        rate, res = cpu_measure(procs, args.n_mol, args.cpu_iters)
        cpu = {"value": rate, "unit": UNIT, "cores": procs, "kind": "port",
               "sample": f"{procs} independent seeded processes x {args.cpu_iters} iterations of the "
                         f"{args.n_mol:,}-molecule model (oracle serial engine, fp64)"}
        if not args.no_cube:
            cube_pool = mp.get_context("spawn").Pool(8)  # started before the first GPU call
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    line = run_gpu(args, rank, world)
    if rank == 0 and not args.no_batch:
        line["batching"] = run_batching(args)
    if rank == 0 and not args.no_serve:
        burst = run_serving(args.serve_rate, args.serve_seconds)
        burst["note"] = ("overload: the configured 50 requests/s offer several times what one GB300 serves, so "
                         "the burst measures a queue draining after arrivals stop")
        line["serving"] = {"overload_burst": burst}
        if args.sustained_seconds > 0:
            sus = run_serving(args.sustained_rate, args.sustained_seconds, plain=False, seed=12)
            cap = burst["plain_sequential"]["molecule_steps_per_s"]
            sus["plain_capacity_molecule_steps_per_s"] = cap
            sus["plain_offered_load_ratio"] = sus["offered_molecule_steps_per_s"] / cap
            sus["note"] = ("sustained arrivals; the plain engine's capacity is measured on the burst's requests run "
                           "one after another: an offered load ratio above 1 means its first-come-first-served "
                           "queue grows without bound at this rate")
            line["serving"]["sustained"] = sus
    if rank == 0 and not args.no_cube:
        line["closed_cube"] = run_closed_cube(args, cube_pool)
    if cube_pool is not None:
        cube_pool.close()
    if rank == 0 and not args.no_precision:
        line["precision"] = run_precision(args)
    if rank == 0:
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
