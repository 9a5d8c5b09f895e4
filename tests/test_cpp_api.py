"""The C++ mirror (include/quantr.hpp): compiles here, its host-side state containers run the
crate's state unit tests here; the simulation cases run on the GPU."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "test_quantr_api.cpp"


def _compile(out: Path, link: bool) -> subprocess.CompletedProcess:
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "include"), str(SRC)]
    if link:
        lib = ROOT / "quantr_gb300" / "lib"
        cmd += ["-L", str(lib), "-lquantr_gpu", f"-Wl,-rpath,{lib}", "-o", str(out)]
    else:
        cmd += ["-c", "-o", str(out)]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_cpp_header_compiles(tmp_path):
    r = _compile(tmp_path / "t.o", link=False)
    assert r.returncode == 0, r.stderr


def test_cpp_state_containers_on_host(tmp_path):
    exe = tmp_path / "test_states_host"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "cpp" / "test_states_host.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "0 failure(s)" in run.stdout


@pytest.mark.gpu
def test_cpp_api_reference_cases_on_gpu(tmp_path, gpu_lib):
    exe = tmp_path / "test_quantr_api"
    r = _compile(exe, link=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "0 failure(s)" in run.stdout
