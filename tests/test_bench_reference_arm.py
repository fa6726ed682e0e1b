"""bench.py --impl reference (the reference arm: the multi-threaded C port of the reference algorithm on
all host cores) needs no GPU: run on the truss lattice, the smallest workload, it prints one JSON line with
the bench contract's keys, its own value as the e2e value with no host-device bytes, and a cpu_baseline
describing the run."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def test_reference_arm_prints_one_contract_line():
    run = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "truss", "--steps", "2", "--warmup", "3"], cwd=ROOT, capture_output=True, text=True,
                         timeout=600, check=True)
    lines = [ln for ln in run.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, run.stdout
    d = json.loads(lines[0])
    assert all(k in d for k in KEYS), set(KEYS) - set(d)
    assert d["impl"] == "reference" and d["metric"] == "elements/s assembled to FP64 CSR"
    assert d["unit"] == "elements/s" and d["higher_is_better"] is True and d["dtype"] == "f64"
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3
    assert d["config"]["nnz"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
