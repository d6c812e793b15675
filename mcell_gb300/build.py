"""Builds the engine library mcell_gb300/_lib/libmcell_gb300.so with nvcc for sm_103a.

Translation units are compiled in parallel:
  mcg_f64.cu    fp64 engine, -fmad=false (bit-identical rounding to the reference's CPU build)
  mcg_f32.cu    fp32 engine (fused multiply-add allowed; checked against the fp64 oracle)
  mcg_setup.cpp host setup (wall constants, wall binning), -ffp-contract=off
  mcg_api.cpp   C ABI (single models)
  mcg_batch.cpp C ABI of batches (replicas) and the batch autotuner
  mcg_serve.cpp C ABI of the serving loop (continuous batching on a worker thread)
  mcg_viz.cpp   visualisation files (ASCII / CellBlender) from device state
  mcg_region.cpp  region releases: object volumes, expression boxes, concentration counts, vacuum choice
  mcg_trace_static.cu  fixed device scratch of mcg_trace_cases_static
Usage: python -m mcell_gb300.build [--force] [-v]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libmcell_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mcell_gb300")


def _units():
    host = ["-Xcompiler", "-fPIC,-ffp-contract=off", "-std=c++17", "-O3"]
    dev = ["-std=c++17", "-O3", "-lineinfo", ARCH, "-Xcompiler", "-fPIC", "--extended-lambda",
           "-Xptxas", "-warn-spills"]
    return [
        ("mcg_f64.cu", dev + ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
        ("mcg_f32.cu", dev),
        ("mcg_trace_static.cu", dev),
        ("mcg_setup.cpp", ["-x", "c++"] + host),
        ("mcg_api.cpp", ["-x", "c++"] + host),
        ("mcg_batch.cpp", ["-x", "c++"] + host),
        ("mcg_serve.cpp", ["-x", "c++"] + host),
        ("mcg_viz.cpp", ["-x", "c++"] + host),
        ("mcg_region.cpp", ["-x", "c++"] + host),
    ]


def _stale(objs) -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    srcs = list(CSRC.glob("*")) + [PKG.parent / "include" / "mcell_gb300.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in srcs)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    units = _units()
    objs = [OUT / (u[0] + ".o") for u in units]
    if not force and not _stale(objs):
        return LIB
    nv = nvcc()

    def compile_one(u):
        src, flags = u
        obj = OUT / (src + ".o")
        cmd = [nv, "-c", str(CSRC / src), "-o", str(obj)] + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"nvcc failed on {src}")
        return obj

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        list(ex.map(compile_one, units))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nv, "-shared", ARCH, "-o", str(tmp)] + [str(o) for o in objs] + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("linking libmcell_gb300.so failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.v))
