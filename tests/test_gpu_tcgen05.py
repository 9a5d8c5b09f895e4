"""The tcgen05 helpers (quantr_gb300/csrc/tc.cuh) on one CTA: tests/cuda/tc_probe.cu multiplies
dyadic 128 x 128 x 16 matrices in TF32 and BF16 through shared-memory descriptors and tensor
memory, and 8-bit integer slices over K = 192 in 12 accumulating BF16 MMAs (sums below 2^24);
the products must equal the host's bit for bit."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def test_tcgen05_probe(tmp_path, gpu_lib):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "tc_probe"
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                        "-I", str(ROOT / "quantr_gb300" / "csrc"),
                        str(ROOT / "tests" / "cuda" / "tc_probe.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.count("PASS") == 3
