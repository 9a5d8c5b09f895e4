"""Host-side logic of the quantr API mirror and the C-ABI library (no GPU needed).

Mirrors the reference's builder/layout tests and its #[should_panic] error tests
(src/circuit.rs:516-597, 715-720, 839-845, 984-991; product_states.rs:274-321).
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from golden import quantr_goldens as G
from quantr_gb300 import Circuit, Gate, ProductState, QuantrError, Qubit, SuperPosition
from quantr_gb300 import _native
from quantr_gb300 import workloads as W
from quantr_gb300.program import OP_DTYPE, lower, tabulate_custom

ROOT = Path(__file__).resolve().parent.parent


def test_pushes_multi_gates():  # src/circuit.rs:535-550
    qc = Circuit(3)
    qc.add_gates([Gate.CNot(2), Gate.CNot(0), Gate.H]).add_gates([Gate.Toffoli(1, 2), Gate.H,
                                                                  Gate.CNot(0)])
    assert qc.get_gates() == G.PUSHED_LAYOUT


def test_pushes_multi_gates_using_vec():  # src/circuit.rs:553-575
    qc = Circuit(3)
    qc.add_gates_with_positions({2: Gate.H, 0: Gate.CNot(2), 1: Gate.CNot(0)}) \
        .add_gates_with_positions({2: Gate.CNot(0), 0: Gate.Toffoli(1, 2), 1: Gate.H})
    assert qc.get_gates() == G.PUSHED_LAYOUT


def test_get_gates_pads_with_identity():  # circuit.rs:94-105
    qc = Circuit(3)
    qc.add_gate(Gate.X, 2)
    assert qc.get_gates() == [Gate.Id, Gate.Id, Gate.X]


@pytest.mark.parametrize("make", [
    lambda: Circuit(3).add_gates([Gate.Id, Gate.Custom(G.example_cnot, [1], "X"), Gate.Id]),
    lambda: Circuit(3).add_gates([Gate.CNot(0), Gate.Id, Gate.Id]),
    lambda: Circuit(3).add_gates_with_positions({2: Gate.H, 0: Gate.CNot(0), 1: Gate.CNot(0)}),
    lambda: Circuit(3).add_gates_with_positions({2: Gate.H, 0: Gate.CNot(2), 1: Gate.CNot(3)}),
    lambda: Circuit(4).add_repeating_gate(Gate.X, [0, 1, 1, 3]),
    lambda: Circuit(3).add_gate(Gate.Custom(G.example_cnot, [0], "NonAscii†"), 1),
    lambda: Circuit(3).add_gate(Gate.X, 1).change_register(
        SuperPosition.from_(ProductState([Qubit.One, Qubit.Zero]))),
    lambda: Circuit(0),
    lambda: Circuit(2).add_gates([Gate.H]),
    lambda: Circuit(2).add_gate(Gate.H, 2),
], ids=["overlapping_custom", "overlapping_control", "overlapping_vec", "control_too_big",
        "repeating_positions", "non_ascii_name", "register_dimension", "zero_wires",
        "column_length", "position_out_of_bounds"])
def test_reference_error_cases_raise(make):
    with pytest.raises(QuantrError):
        make()


def test_product_state_ordering():  # product_states.rs:274-321
    assert ProductState.binary_basis(6, 3) == ProductState([Qubit.One, Qubit.One, Qubit.Zero])
    assert ProductState([1, 0, 1]).comp_basis() == 5
    assert ProductState([1, 1, 1]).comp_basis() == 7
    assert ProductState([1, 0]).comp_basis() == 2
    assert ProductState([1, 0, 1, 1]).comp_basis() == 11
    p = ProductState([1, 1, 1])
    p.insert_qubits([Qubit.Zero, Qubit.Zero], [0, 2])
    assert p == ProductState([0, 1, 0])
    assert str(ProductState([0, 1])) == "01"


def test_superposition_constructors_and_checks():  # super_positions.rs:403-544
    s = SuperPosition.new(2)
    s.set_amplitudes([0, 2 ** -0.5, -1j * 2 ** -0.5, 0])
    assert s.get_amplitude_from_state(ProductState([Qubit.Zero, Qubit.One])) == pytest.approx(2 ** -0.5)
    assert s.get_amplitude(4) is None
    with pytest.raises(QuantrError):
        s.set_amplitudes([0, 0.5, 0, -0.5j])
    with pytest.raises(QuantrError):
        s.get_amplitude_from_state(ProductState([0, 1, 1]))
    with pytest.raises(QuantrError):
        SuperPosition.new_with_hash_amplitudes({ProductState([0, 1]): 2 ** -0.5,
                                                ProductState([1, 0, 1]): -1j * 2 ** -0.5})
    hm = SuperPosition.new_with_amplitudes([0, 2 ** -0.5, 2 ** -0.5, 0]).to_hash_map()
    assert set(map(str, hm)) == {"01", "10"}
    it = list(SuperPosition.new_with_amplitudes([0, 2 ** -0.5, 2 ** -0.5, 0]))
    assert str(it[1][0]) == "01" and it[1][1] == pytest.approx(2 ** -0.5)


def test_lowering_positions_follow_counter_mod_n():  # simulation.rs:37-56
    qc = Circuit(3)
    qc.add_gates([Gate.H, Gate.Id, Gate.Rz(0.25)]).add_gate(Gate.CNot(0), 2) \
        .add_gate(Gate.Toffoli(2, 0), 1).add_gate(Gate.CRk(3, 1), 0)
    prog = lower(qc.get_gates(), 3)
    kinds = [_native.KINDS[k] for k in prog.ops["kind"]]
    assert kinds == ["H", "Rz", "CNot", "Toffoli", "CRk"]
    assert list(prog.ops["target"]) == [0, 2, 2, 1, 0]
    assert list(prog.ops["n_controls"]) == [0, 0, 1, 2, 1]
    assert prog.ops["controls"][3][:2].tolist() == [2, 0]
    assert prog.ops["k"][4] == 3 and prog.ops["param"][1] == 0.25


def test_custom_tabulation_columns_and_none():
    block, none = tabulate_custom(G.example_cnot, 2)
    assert none.tolist() == [1, 1, 0, 0]
    assert np.array_equal(block[2], [0, 0, 0, 1]) and np.array_equal(block[3], [0, 0, 1, 0])
    with pytest.raises(QuantrError):
        tabulate_custom(lambda p: SuperPosition.new_with_amplitudes_unchecked([1, 0]), 2)


def test_workloads_are_deterministic_and_api_consistent():
    a = W.brickwork_qft(n=6, layers=3, seed=9)
    b = W.brickwork_qft(n=6, layers=3, seed=9)
    assert a.ops.tobytes() == b.ops.tobytes()
    c = lower(W.brickwork_qft_circuit(6, layers=3, seed=9).get_gates(), 6)
    assert c.ops.tobytes() == a.ops.tobytes()
    assert len(W.brickwork_qft(n=30).ops) == 20 * 90 + sum(1 for l in range(20)
                                                           for _ in range(l % 2, 29, 2)) + 30 + 435 + 15
    r = W.random_columns(n=12, seed=1)
    assert len(r.ops) > 40 * 12


def test_op_record_layout_matches_header():
    hdr = (ROOT / "include" / "qgpu.h").read_text()
    assert "QGPU_MAX_OP_WIRES 10" in hdr
    assert OP_DTYPE.itemsize == C.sizeof(_native.QgpuOp) == 80


def test_library_loads_and_exports_every_declared_symbol():
    """The C-ABI library loads without a GPU and exports every function of include/*.h."""
    lib = _native.load()
    declared = set()
    for h in (ROOT / "include").glob("*.h"):
        declared |= set(re.findall(r"^\s*(?:int|const char\s*\*|uint64_t|void\s*\*?)\s*(qgpu_\w+)\s*\(",
                                   h.read_text(), re.M))
    assert "qgpu_apply_program" in declared and "qgpu_measure" in declared
    for name in sorted(declared):
        assert hasattr(lib, name), f"{name} not exported"
    assert set(_native.exported_symbols()) <= declared | set()


def test_no_oracle_in_product_package():
    """The product package never imports or links the oracle."""
    pat = re.compile(r"(import\s+oracle|from\s+oracle|liboracle|quantr_oracle|oracle_simulate)")
    for p in (ROOT / "quantr_gb300").rglob("*"):
        if p.suffix in (".py", ".cu", ".cuh", ".cpp", ".h"):
            assert not pat.search(p.read_text()), p


def _message(make) -> str:
    with pytest.raises(QuantrError) as e:
        make()
    return e.value.message


def test_validation_messages_print_gates_as_the_crate_does():  # circuit.rs:272-293
    # repeated nodes are found before a node on the gate's own wire
    assert _message(lambda: Circuit(3).add_gates([Gate.CNot(0), Gate.Id, Gate.Id])) == \
        "The gate, CNot(0), has a control node that equals the gate's position 0."
    assert _message(lambda: Circuit(3).add_gates([Gate.Toffoli(0, 0), Gate.Id, Gate.Id])) == \
        "The gate, Toffoli(0, 0), has overlapping control nodes."
    assert _message(lambda: Circuit(3).add_gates_with_positions(
        {2: Gate.H, 0: Gate.CNot(2), 1: Gate.CNot(3)})) == \
        "The control node at position 3, is greater than the umnber of qubits 3."


def test_gate_debug_format():  # `{:?}` of gate.rs:18-45
    assert repr(Gate.H) == "H"
    assert repr(Gate.Rx(0.5)) == "Rx(0.5)"
    assert repr(Gate.Phase(1.0)) == "Phase(1.0)"
    assert repr(Gate.Rz(1e-5)) == "Rz(1e-5)"
    assert repr(Gate.CR(2.0, 1)) == "CR(2.0, 1)"
    assert repr(Gate.CRk(3, 1)) == "CRk(3, 1)"
    assert repr(Gate.Toffoli(0, 2)) == "Toffoli(0, 2)"
    r = repr(Gate.Custom(G.example_cnot, [0, 1], 'q"x'))
    assert r.startswith("Custom(0x") and r.endswith(', [0, 1], "q\\"x")')


def test_f64_in_messages_as_rust_prints_it():
    from quantr_gb300.errors import rust_debug_f64, rust_debug_str, rust_display_f64

    assert [rust_display_f64(x) for x in (2.0, 0.5, 1e-7, 0.1 + 0.2, -0.0, 1e21)] == \
        ["2", "0.5", "0.0000001", "0.30000000000000004", "-0", "1000000000000000000000"]
    assert [rust_debug_f64(x) for x in (1.0, 0.5, 1e-5, -2.5e-7, 1e16, 1234.5)] == \
        ["1.0", "0.5", "1e-5", "-2.5e-7", "1e16", "1234.5"]
    assert rust_debug_str('a"b\\c\n') == '"a\\"b\\\\c\\n"'
    # super_positions.rs:122 prints the total with `{}`
    st = {ProductState([Qubit.Zero, Qubit.One]): 2 ** -0.5,
          ProductState([Qubit.One, Qubit.Zero]): -0.5j * 2 ** -0.5}
    assert _message(lambda: SuperPosition.new_with_hash_amplitudes(st)).startswith(
        "The total sum of the absolute square of all amplitudes, 0.625")
    s = SuperPosition.new(2)
    assert _message(lambda: s.get_amplitude_from_state(ProductState([0, 1, 1]))).startswith(
        'Unable to retreive product state, |"011"> with dimension 3.')


def test_progress_log_format(capsys):  # simulation.rs:32-34, 183-200
    from quantr_gb300.circuit import _print_log

    _print_log([Gate.H, Gate.Id, Gate.CNot(0), Gate.Id, Gate.Rz(0.5), Gate.Id], 3)
    _print_log([Gate.Id, Gate.X], 2)
    assert capsys.readouterr().out == (
        "Starting circuit simulation...\n"
        "Applying H on wire 0 # 1/6 \n"
        "Applying CNot(0) on wire 2 # 3/6 \n"
        "Applying Rz(0.5) on wire 1 # 5/6 \n"
        "Starting circuit simulation...\n"
        "Applying X on wire 1 # 2/2 \n"
        "Finished circuit simulation.\n")


def test_abi_rejects_null_handles_and_bad_sizes():
    """Every entry point taking a handle returns QGPU_ERR_INVALID on NULL with a message naming
    itself (qgpu_destroy(NULL) is a no-op, as free(NULL)); qgpu_create checks its size and
    precision before touching a device. No call here reaches the GPU."""
    lib = _native.load()
    checked = 0
    for name, (res, args) in _native._EXPORTS.items():
        if not args or args[0] is not C.c_void_p:
            continue
        vals = [1 if a is C.c_uint32 else 0 if a in (C.c_int, C.c_size_t, C.c_uint64, C.c_double)
                else None for a in args]
        r = getattr(lib, name)(*vals)
        if name == "qgpu_destroy":
            assert r == 0
        elif name == "qgpu_stream":
            assert r is None
        elif name == "qgpu_launch_count":
            assert r == 0
        else:
            assert r == _native.QGPU_ERR_INVALID, name
            assert lib.qgpu_last_error().decode().startswith(name + ":"), name
            checked += 1
    assert checked >= 18
    h = C.c_void_p()
    for n, prec in ((0, _native.QGPU_C128), (41, _native.QGPU_C128), (3, 7)):
        assert lib.qgpu_create(n, prec, C.byref(h)) == _native.QGPU_ERR_INVALID
        assert h.value is None
    assert lib.qgpu_create(0, _native.QGPU_C128, C.byref(h)) == _native.QGPU_ERR_INVALID
    assert b"1..40 qubits" in lib.qgpu_last_error()
    assert lib.qgpu_create(3, _native.QGPU_C128, None) == _native.QGPU_ERR_INVALID


def test_no_cpu_fallback_without_a_gpu():
    """On a machine without a GPU the engine fails loudly: qgpu_create returns a CUDA error with
    a message, and the Python API raises QuantrError instead of simulating on the host."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _native.load()
    h = C.c_void_p()
    st = lib.qgpu_create(3, _native.QGPU_C128, C.byref(h))
    assert st == _native.QGPU_ERR_CUDA and h.value is None
    assert lib.qgpu_last_error()
    with pytest.raises(QuantrError):
        Circuit(2).add_gate(Gate.H, 0).simulate()


def test_superposition_measure_is_the_crate_rule():  # super_positions.rs:332-342
    """The first i with u < the running sum of |a_i|^2 (sequential f64 adds), None past the total;
    checked against the literal loop, u on and next to every cumulative value."""
    rng = np.random.default_rng(8)
    for n in (1, 3, 6):
        a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        a[rng.random(a.size) < 0.3] = 0
        a /= np.linalg.norm(a) * (1.0 if n != 3 else 1.2)  # n = 3: unnormalised, total < 1
        sp = SuperPosition.new_with_amplitudes_unchecked(a)
        cum, c = [], 0.0
        for x in a:
            c += x.real * x.real + x.imag * x.imag
            cum.append(c)
        us = list(rng.random(200)) + cum + [np.nextafter(v, 0) for v in cum] + [0.0, 0.999999]
        for u in us:
            want = next((i for i, v in enumerate(cum) if u < v), None)
            got = sp.measure(u)
            if want is None:
                assert got is None
            else:
                assert got == ProductState.binary_basis(want, n)


def test_crate_doc_examples_states():
    """The assertions of the crate's rustdoc examples for the state types (product_states.rs,
    product_states_iter.rs, qubit.rs, super_positions.rs, super_position_iter.rs, circuit.rs)."""
    r = 2 ** -0.5
    prod = ProductState([Qubit.One, Qubit.Zero])                       # product_states.rs:55-62
    assert prod.get(1) == Qubit.Zero and prod.get(2) is None
    assert prod.get_qubits() == [Qubit.One, Qubit.Zero]                 # :72-78
    prod.get_mut_qubits()[1] = Qubit.One                                # :90-97
    assert prod.get_qubits() == [Qubit.One, Qubit.One]
    assert ProductState([Qubit.Zero, Qubit.One, Qubit.Zero]).num_qubits() == 3   # :127-133
    p = ProductState([Qubit.One, Qubit.Zero, Qubit.One])                # :145-152
    p.invert_digit(1)
    assert p.get_qubits() == [Qubit.One, Qubit.One, Qubit.One]
    assert ProductState([Qubit.Zero, Qubit.Zero]).kronecker_prod(Qubit.One).get_qubits() == \
        [Qubit.Zero, Qubit.Zero, Qubit.One]                             # :170-178
    assert str(ProductState([Qubit.Zero, Qubit.One])) == "01"           # :221-227
    assert ProductState.from_(Qubit.One).get_qubits() == [Qubit.One]    # :245-251
    assert list(ProductState([Qubit.One, Qubit.Zero, Qubit.Zero])) == \
        [Qubit.One, Qubit.Zero, Qubit.Zero]                             # product_states_iter.rs:17-27
    assert Qubit.Zero.kronecker_prod(Qubit.One).get_qubits() == [Qubit.Zero, Qubit.One]  # qubit.rs:27-33
    s = SuperPosition.new(2)                                            # super_positions.rs:33-39
    assert list(s.get_amplitudes()) == [1, 0, 0, 0]
    assert list(SuperPosition.new_with_amplitudes([1, 0, 0, 0]).get_amplitudes()) == [1, 0, 0, 0]
    h = SuperPosition.new_with_hash_amplitudes({ProductState([Qubit.Zero, Qubit.One]): 1.0})
    assert list(h.get_amplitudes()) == [0, 1, 0, 0]                     # :96-103
    assert SuperPosition.new_with_amplitudes([0, 1, 0, 0]).get_amplitude(1) == 1   # :137-143
    assert s.get_num_qubits() == 2 and s.get_dimension() == 4           # :152-173
    assert SuperPosition.new_with_amplitudes([0, 1, 0, 0]).get_amplitude_from_state(
        ProductState([Qubit.Zero, Qubit.One])) == 1                     # :197-205
    t = SuperPosition.new(2)
    t.set_amplitudes([0, 1, 0, 0])                                      # :219-227
    assert list(t.get_amplitudes()) == [0, 1, 0, 0]
    u = SuperPosition.new(2)
    u.set_amplitudes_from_states({ProductState([Qubit.Zero, Qubit.One]): 1.0})   # :259-268
    assert list(u.get_amplitudes()) == [0, 1, 0, 0]
    assert SuperPosition.new(2).to_hash_map() == {ProductState([Qubit.Zero, Qubit.Zero]): 1}  # :303-313
    it = list(SuperPosition.new_with_amplitudes([0, r, r, 0]))          # super_position_iter.rs:18-37
    assert it == [(ProductState([Qubit.Zero, Qubit.Zero]), 0), (ProductState([Qubit.Zero, Qubit.One]), r),
                  (ProductState([Qubit.One, Qubit.Zero]), r), (ProductState([Qubit.One, Qubit.One]), 0)]
    qc = Circuit(3)                                                     # circuit.rs:66-71, 94-101
    assert qc.get_num_qubits() == 3
    qc.add_gate(Gate.X, 2)
    assert qc.get_gates() == [Gate.Id, Gate.Id, Gate.X]


def test_histogram_behaves_as_the_crate_hashmap():
    """measure_all's HashMap<ProductState, usize>, backed by the sampler's sorted arrays: lookups,
    membership (keys of another dimension are absent), iteration, equality with a dict."""
    from quantr_gb300.circuit import Histogram

    h = Histogram(np.array([1, 5, 30], np.uint64), np.array([7, 2, 1], np.uint64), 5)
    k5 = ProductState.binary_basis(5, 5)
    assert len(h) == 3 and h[k5] == 2 and k5 in h
    assert ProductState([1, 0, 1]) not in h          # |101>: 3 qubits, not |00101>
    assert ProductState.binary_basis(4, 5) not in h and "00101" not in h
    with pytest.raises(KeyError):
        h[ProductState.binary_basis(2, 5)]
    assert [str(k) for k in h] == ["00001", "00101", "11110"]
    assert dict(h) == {ProductState.binary_basis(1, 5): 7, k5: 2, ProductState.binary_basis(30, 5): 1}
    assert h == dict(h) and h.total() == 10
    assert h.get(ProductState.binary_basis(3, 5), 0) == 0


def test_builder_rejects_wires_outside_the_register():
    """Positions and control nodes are usize in quantr: a negative one is rejected like one past
    the register, never wrapped round to the last wire; repeated positions report the list."""
    def msg(make):
        with pytest.raises(QuantrError) as e:
            make()
        return e.value.message

    assert msg(lambda: Circuit(3).add_gate(Gate.H, -1)) == \
        "The position, -1, is out of bounds for the circuit with 3 qubits."
    assert msg(lambda: Circuit(3).add_gate(Gate.CNot(-1), 0)) == \
        "The control node at position -1, is greater than the umnber of qubits 3."
    assert msg(lambda: Circuit(3).add_repeating_gate(Gate.H, [-1])).startswith("The position, -1,")
    assert msg(lambda: Circuit(3).add_repeating_gate(Gate.H, [0, 3])).startswith("The position, 3,")
    assert msg(lambda: Circuit(4).add_repeating_gate(Gate.X, [0, 1, 1, 3])) == \
        "Attempted to add more than one gate onto a single wire. The positions in [0, 1, 1, 3] " \
        "must all differ."
    assert Circuit(3).add_repeating_gate(Gate.H, [2, 0]).get_gates() == [Gate.H, Gate.Id, Gate.H]
