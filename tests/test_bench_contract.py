"""The reference arm of bench.py (the oracle's serial engine on the host cores; no GPU):
one JSON line with the contract's keys, on a small sample; under a multi-rank launch
only rank 0 prints it."""
import json
import os
import subprocess
import sys

from tests import harness as H

CMD = [sys.executable, str(H.ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
       "--n-mol", "20000", "--cpu-procs", "2"]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run(CMD, capture_output=True, text=True, timeout=300, cwd=H.ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert "20,000 molecules" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] == 2 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run(CMD, capture_output=True, text=True, timeout=300, cwd=H.ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [x for x in r.stdout.splitlines() if x.startswith("{")]
