"""The adjoint sweep's host-side algebra checked without a GPU (tests/cpp/adjoint_host.cpp):
inverse_op against the library's own tabulation for every gate kind, and the Pauli-sum
coefficients of single-wire runs (pauli_run, quantr_gb300/csrc/plan.cpp) against central
differences of the energy (h = 1e-6; bar 1e-8, measured about 1e-9), the gather tables of
CNot / X / Swap runs (affine_tables, the k_linperm pass) against the gates applied one by one
(exact), and the wire-to-pass partition of the grouped sweep (adj_group_passes: every wire once,
tiles of at most 11 bits holding bits 0..4, the expected pass counts)."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_adjoint_host_algebra(tmp_path):
    exe = tmp_path / "adjoint_host"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "cpp" / "adjoint_host.cpp"),
                        str(ROOT / "quantr_gb300" / "csrc" / "plan.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "fails 0" in run.stdout
