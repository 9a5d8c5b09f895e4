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


def test_cpp_and_python_mirrors_lower_alike(tmp_path):
    """The same circuit (every gate kind, Custom gates with None entries and a non-unitary
    complex image) lowered by the C++ mirror (tests/cpp/lower_dump.cpp) and by the Python
    mirror gives byte-identical gate programs: the same qgpu_op records, Custom block doubles
    and None flags."""
    import numpy as np

    from golden import quantr_goldens as G
    from quantr_gb300 import Circuit, Gate, ProductState, Qubit, SuperPosition
    from quantr_gb300.program import OP_DTYPE, lower

    exe = tmp_path / "lower_dump"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "cpp" / "lower_dump.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    f = [tmp_path / n for n in ("ops.bin", "mats.bin", "none.bin")]
    run = subprocess.run([str(exe)] + [str(x) for x in f], capture_output=True, text=True,
                         timeout=60)
    assert run.returncode == 0, run.stderr

    def scaled(p: ProductState):
        if p.get_qubits()[0] == Qubit.Zero:
            # complex(0, -0.3), not -0.3j (whose real part is -0.0)
            return SuperPosition.new_with_amplitudes_unchecked([complex(0.6, 0.1), complex(0, -0.3)])
        return SuperPosition.new_with_amplitudes_unchecked([0, 0])

    qc = Circuit(5)
    qc.add_repeating_gate(Gate.H, [0, 1, 2, 3, 4])
    qc.add_gates([Gate.X, Gate.Y, Gate.Z, Gate.S, Gate.Sdag])
    qc.add_gates([Gate.T, Gate.Tdag, Gate.X90, Gate.Y90, Gate.MX90])
    qc.add_gates([Gate.MY90, Gate.Rx(0.25), Gate.Ry(-1.5), Gate.Rz(3.0), Gate.Phase(0.7)])
    qc.add_gate(Gate.CR(1.1, 0), 3).add_gate(Gate.CRk(3, 4), 1).add_gate(Gate.CZ(2), 0)
    qc.add_gate(Gate.CY(1), 4).add_gate(Gate.CNot(0), 2).add_gate(Gate.Swap(4), 1)
    qc.add_gate(Gate.Toffoli(0, 4), 2)
    qc.add_gate(Gate.Custom(G.cccnot, [0, 1, 2], "X"), 3)
    qc.add_gate(Gate.Custom(G.example_cnot, [4], "X"), 0)
    qc.add_gate(Gate.Custom(scaled, [], "P"), 2)
    qc.add_gates([Gate.Id, Gate.CNot(4), Gate.Id, Gate.H, Gate.Rx(0.5)])
    prog = lower(qc.get_gates(), 5)

    ops = np.fromfile(f[0], dtype=OP_DTYPE)
    assert ops.size == prog.ops.size == 33
    assert ops.tobytes() == np.ascontiguousarray(prog.ops).tobytes()
    assert np.fromfile(f[1], dtype=np.float64).tobytes() == \
        np.ascontiguousarray(prog.mats, dtype=np.float64).tobytes()
    assert np.fromfile(f[2], dtype=np.uint8).tobytes() == \
        np.ascontiguousarray(prog.none, dtype=np.uint8).tobytes()
