"""bench.py's reference arm runs on the host alone (the CPU oracle), so its
JSON line is checked here: one line with the contract's keys, the oracle as
the reference implementation, and an e2e block without device copies."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


import pytest


@pytest.mark.parametrize("workload,size", [("anderson", 10), ("laplace", 8), ("tightbinding", 6), ("fem", 12)])
def test_reference_arm_json_line(workload, size):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", workload,
                        "--size", str(size), "--steps", "1", "--warmup", "3"], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    # standard output carries the result line alone (the solver's own messages go to stderr)
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 1 and lines[0].startswith("{"), r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 1 and d["warmup"] == 3
    assert d["value"] > 0 and d["higher_is_better"] is False
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert "workload" in d["config"]


@pytest.mark.parametrize("workload,size,neig", [("tightbinding", 8, 8), ("fem", 16, 6)])
def test_cpu_baseline_with_the_oracles_own_factor(workload, size, neig):
    """The CPU-baseline leg of the complex and generalized workloads (whose
    factors are not exported): the oracle factors the same matrix itself and
    its per-MATVEC time is scaled to the GPU solve's MATVEC count."""
    sys.path.insert(0, ROOT)
    import bench
    old = sys.argv
    try:
        sys.argv = ["bench.py", "--workload", workload, "--size", str(size), "--neig", str(neig),
                    "--cpu-seconds", "1"]
        args = bench.parse()
    finally:
        sys.argv = old
    w = bench.make_workload(args)
    cb = bench.cpu_baseline_own_factor(args, w, 300)
    assert cb["kind"] == "port" and cb["cores"] == 1 and cb["unit"] == "s"
    assert cb["value"] > 0 and "MATVECs" in cb["sample"]
