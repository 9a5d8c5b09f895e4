"""The tensor-core double pair pass (quantr_gb300/csrc/pair_tc.cu) checked on the host:
tests/cpp/pair_tc_host.cu builds the kernel's B operand with the library's own image builder and
emulates the kernel's arithmetic (48-bit fixed-point slices, the 26 slice products of weight
>= 4 as exact integer sums, recombination and rescaling) against the complex128 product.

Bar: max |emulated - exact| <= 1e-12 of the tile's largest amplitude (measured 2-3e-14)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_pair_tc_arithmetic_on_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path / "pair_tc_host"
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                        "-I", str(ROOT / "quantr_gb300" / "csrc"),
                        str(ROOT / "tests" / "cpp" / "pair_tc_host.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "fails 0" in run.stdout
