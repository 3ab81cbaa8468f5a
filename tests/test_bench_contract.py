"""The bench line's contract, on the CPU: the reference arm (the oracle
restatement under OpenMP on the host cores) prints one JSON line with the
keys the GPU arm's line shares, on a small mesh."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def run_bench(*args):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True, timeout=300,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_reference_arm_line():
    d = run_bench("--impl", "reference", "--n", "12", "--steps", "2", "--warmup", "1")
    assert d["impl"] == "reference" and d["unit"] == "cycles/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert abs(d["ms_per_step"] - 1e3 / d["value"]) <= 1e-3 * d["ms_per_step"] + 1e-3
    assert d["dtype"] == "f64" and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["config"]["workload"].startswith("12^3") and "fit in L2" in d["config"]["l2"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["e2e"]["d2h_bytes_per_step"] == 0


def test_help_lists_the_forms():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True, timeout=60,
                       cwd=ROOT)
    assert r.returncode == 0
    for flag in ("--precision", "--increment", "--mode", "--impl", "--loops-forms"):
        assert flag in r.stdout
