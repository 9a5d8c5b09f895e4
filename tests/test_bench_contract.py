"""bench.py's reference arm on the host: one JSON line with the keys of the benchmark contract
(the line of our own arm needs a GPU and is covered by the GPU runs)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--ref-n", "10", "--ref-budget", "0.5"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 3
    assert line["higher_is_better"] is True and line["n_gpus"] == 1
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    # every host core runs one independent single-threaded simulation (quantr has no threads)
    assert cb["value"] == line["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert cb["cpu"]["nproc"] >= cb["cores"] and cb["single_core_value"] > 0
    assert cb["unit"] == line["unit"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
