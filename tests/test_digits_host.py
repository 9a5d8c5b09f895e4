"""The digit pair passes (quantr_gb300/csrc/digits.cu) checked on the host:
tests/cpp/digits_host.cu runs the library's own image builder (matrix digits in the B operand's
layout, carry constants), the byte permutes that form the A operand, the MMA step table and the
carry chain, with exact integer sums in place of the tensor cores' exact F32 accumulation, against
an extended-precision product. Random 16 x 16 unitaries and Kronecker products of 4 x 4 blocks
with slot permutations; tiles of unit norm over many magnitudes, single amplitudes of modulus 1,
the zero tile.

Bar: |emulated - exact| <= 4 units of 2^-54 per real (measured 0.67); an adversarial matrix whose
digit sums could leave the exact range is rejected."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_digit_pass_arithmetic_on_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path / "digits_host"
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                        "-I", str(ROOT / "quantr_gb300" / "csrc"), "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "cpp" / "digits_host.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "fails 0" in run.stdout and "big_rejected 1" in run.stdout
