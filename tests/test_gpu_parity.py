"""GPU parity: libquantr_gpu against the oracle and the reference's own known answers.

Bars (written per test):
  * QGPU_MODE_EXACT (complex128): amplitudes equal the oracle's value for value (np.array_equal;
    only the sign of a zero may differ).
  * QGPU_MODE_FAST / QGPU_MODE_F64 (complex128): max |a_gpu - a_oracle| <= 1e-12.
  * complex64: fidelity 1 - |<psi64|psi128>|^2 <= 1e-8 and max |delta a| <= 1e-5.
  * shots: index-for-index equal to the oracle's linear-scan rule for the same uniforms, except
    where u lies within 1e-12 of a cumulative boundary; seeded histograms pass a chi-square test
    against the oracle's |a|^2.
"""
import math

import numpy as np
import pytest

from golden import quantr_goldens as G
from quantr_gb300 import Circuit, Gate, QuantrError, SuperPosition, set_default_backend
from quantr_gb300 import _native as nat
from quantr_gb300 import workloads as W
from quantr_gb300.program import ProgramBuilder, lower

pytestmark = pytest.mark.gpu

TOL_FAST = 1e-12
MODES = {"exact": nat.QGPU_MODE_EXACT, "fast": nat.QGPU_MODE_FAST, "f64": nat.QGPU_MODE_F64}


def run_gpu(prog, mode, precision=nat.QGPU_C128, reg=None):
    h = nat.Handle(prog.n, precision, MODES[mode] if isinstance(mode, str) else mode)
    if reg is not None:
        h.upload(reg)
    h.apply(prog.ops, prog.mats, prog.none)
    out = h.download()
    h.close()
    return out


@pytest.fixture(autouse=True)
def _lib(gpu_lib):
    yield
    set_default_backend(precision="c128", mode="fast")


@pytest.mark.parametrize("mode", ["exact", "fast", "f64"])
@pytest.mark.parametrize("case", G.AMPLITUDE_CASES, ids=[c[0] for c in G.AMPLITUDE_CASES])
def test_reference_goldens_on_gpu(case, mode):
    name, builder, expected, tol, cite = case
    set_default_backend(mode=mode)
    qc = builder()
    out = qc.simulate().get_state().take().get_amplitudes()
    assert np.max(np.abs(out - expected)) < tol, cite


def test_exact_mode_equals_oracle_cfg1(oracle):
    """12-qubit random columns (the CPU-runnable config): value-for-value equal."""
    prog = W.random_columns(n=12, seed=1)
    ref = oracle.simulate(prog, engine=oracle.HASHMAP)
    out = run_gpu(prog, "exact")
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_exact_mode_equals_oracle_random(oracle, seed):
    prog = W.random_columns(n=9, columns=25, seed=seed)
    assert np.array_equal(run_gpu(prog, "exact"), oracle.simulate(prog, engine=oracle.DENSE))


def test_exact_mode_equals_oracle_brickwork(oracle):
    prog = W.brickwork_qft(n=12, layers=6, seed=2)
    assert np.array_equal(run_gpu(prog, "exact"), oracle.simulate(prog, engine=oracle.DENSE))


def test_exact_mode_customs_equal_oracle(oracle):
    prog = lower(G.x3sudoko_circuit().get_gates(), 10)
    assert np.array_equal(run_gpu(prog, "exact"), oracle.simulate(prog, engine=oracle.HASHMAP))


@pytest.mark.parametrize("mode", ["fast", "f64"])
def test_fused_modes_within_tolerance_cfg1(oracle, mode):
    prog = W.random_columns(n=12, seed=1)
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    assert np.max(np.abs(run_gpu(prog, mode) - ref)) <= TOL_FAST


_BRICKWORK_REF = {}


def _brickwork_ref(oracle, n):
    """The oracle's amplitudes for the headline family at n qubits (threaded dense engine, equal
    value for value to the dense engine), computed once per session."""
    if n not in _BRICKWORK_REF:
        prog = W.brickwork_qft(n=n, layers=20, seed=2)
        _BRICKWORK_REF[n] = (prog, oracle.simulate(prog, engine=oracle.DENSE_PAR))
    return _BRICKWORK_REF[n]


@pytest.mark.parametrize("mode", ["fast", "f64", "exact"])
@pytest.mark.parametrize("n", [5, 11, 16, 20, 22])
def test_fused_modes_brickwork_qft(oracle, mode, n):
    """The 30-qubit headline family (20 brickwork layers + QFT + swaps) against the oracle up to
    22 qubits: fused modes within 1e-12 max-abs, exact mode value for value."""
    prog, ref = _brickwork_ref(oracle, n)
    out = run_gpu(prog, mode)
    if mode == "exact":
        assert np.array_equal(out, ref)
    else:
        assert np.max(np.abs(out - ref)) <= TOL_FAST


def test_compare_registers_on_the_device(oracle):
    """qgpu_compare (max |a - b| and <a|b> without a download) against the same figures from
    downloaded amplitudes, for complex128 fast vs exact and complex128 vs complex64."""
    prog, _ = _brickwork_ref(oracle, 16)
    hs = [nat.Handle(16, p, m) for p, m in ((nat.QGPU_C128, nat.QGPU_MODE_FAST),
                                            (nat.QGPU_C128, nat.QGPU_MODE_EXACT),
                                            (nat.QGPU_C64, nat.QGPU_MODE_FAST))]
    outs = []
    for h in hs:
        h.apply(prog.ops, prog.mats, prog.none)
        outs.append(h.download())
    for i, j in ((0, 1), (1, 0), (0, 2), (2, 1)):
        mx, inner = hs[i].compare(hs[j])
        want_mx = np.max(np.abs(outs[i] - outs[j]))
        want_in = np.vdot(outs[i], outs[j])
        assert abs(mx - want_mx) <= 1e-15 + 1e-12 * want_mx
        assert abs(inner - want_in) <= 1e-12
    assert hs[0].compare(hs[1])[0] <= TOL_FAST
    with pytest.raises(QuantrError):
        hs[0].compare(nat.Handle(15))
    for h in hs:
        h.close()


@pytest.mark.parametrize("mode", ["exact", "fast", "f64"])
def test_every_gate_on_every_wire(oracle, mode):
    """Exhaustive sweep: each gate kind on each target, controls above and below the target,
    on a random register (bit-mask indexing must be exact for every position)."""
    n = 6
    rng = np.random.default_rng(5)
    reg = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    reg /= np.linalg.norm(reg)
    b = ProgramBuilder(n)
    for t in range(n):
        for name in ("H", "X", "Y", "Z", "S", "Sdag", "T", "Tdag", "X90", "Y90", "MX90", "MY90"):
            b.add(name, t)
        for name in ("Rx", "Ry", "Rz", "Phase"):
            b.add(name, t, (), param=0.3 + t)
        for c in range(n):
            if c == t:
                continue
            b.add("CNot", t, (c,))
            b.add("CY", t, (c,))
            b.add("CZ", t, (c,))
            b.add("Swap", t, (c,))
            b.add("CR", t, (c,), param=0.7 * c - t)
            b.add("CRk", t, (c,), k=1 + (c + t) % 5)
            c2 = (c + 1 + t) % n
            if c2 not in (c, t):
                b.add("Toffoli", t, (c, c2))
    prog = b.build()
    ref = oracle.simulate(prog, reg, engine=oracle.DENSE)
    out = run_gpu(prog, mode, reg=reg)
    if mode == "exact":
        assert np.array_equal(out, ref)
    else:
        assert np.max(np.abs(out - ref)) <= TOL_FAST


@pytest.mark.parametrize("precision", [nat.QGPU_C128, nat.QGPU_C64])
def test_commuting_cx_runs(oracle, precision):
    """Runs of commuting controlled-X gates (bricks with controls above and below the targets,
    Toffolis, bare X) applied as one index involution per run."""
    n = 11
    rng = np.random.default_rng(8)
    reg = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    reg /= np.linalg.norm(reg)
    b = ProgramBuilder(n)
    for i in range(0, n - 1, 2):
        b.add("CNot", i + 1, (i,))         # control one wire above: control bit = target bit + 1
    b.add("Ry", 3, (), param=0.4)
    for i in range(1, n - 1, 2):
        b.add("CNot", i, (i + 1,))         # control below the target
    b.add("Toffoli", 10, (0, 4))
    b.add("X", 2)
    b.add("Toffoli", 6, (8, 1))
    b.add("H", 5)
    b.add("X", 0); b.add("CNot", 3, (7,)); b.add("X", 9); b.add("Toffoli", 4, (2, 6))
    b.add("T", 1)
    for i in range(4):                     # QFT-style swaps, then controlled-X on other wires
        b.add("Swap", i, (n - 1 - i,))
    b.add("CNot", 5, (4,))
    b.add("Swap", 6, (5,))                  # overlaps the CNot: starts a new run
    prog = b.build()
    ref = oracle.simulate(prog, reg, engine=oracle.DENSE)
    out = run_gpu(prog, "fast", precision=precision, reg=reg)
    tol = TOL_FAST if precision == nat.QGPU_C128 else 1e-6
    assert np.max(np.abs(out - ref)) <= tol


@pytest.mark.parametrize("variant", ["1", "2"])
@pytest.mark.parametrize("n", [11, 13, 16])
def test_double_pair_passes_on_tensor_cores(oracle, monkeypatch, n, variant):
    """k_pair2_tc (QGPU_PAIR2_TC=1) and its warp-specialised form k_pair2_ws (=2): the double
    pair passes of the brickwork + QFT family on the tensor cores through 8-bit fixed-point
    slices; complex128 within the fused-mode bar."""
    monkeypatch.setenv("QGPU_PAIR2_TC", variant)
    prog = W.brickwork_qft(n=n, layers=20, seed=7)
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    h = nat.Handle(n, nat.QGPU_C128, nat.QGPU_MODE_FAST)
    h.set_profiling(True)
    h.apply(prog.ops, prog.mats, prog.none)
    out = h.download()
    prof = h.profile(reset=True)
    h.close()
    assert ("k_pair2_ws" if variant == "2" else "k_pair2_tc") in prof  # the tensor-core kernel ran
    assert np.max(np.abs(out - ref)) <= TOL_FAST
    assert abs(np.sum(np.abs(out) ** 2) - 1.0) <= 1e-12


@pytest.mark.parametrize("variant", ["1", "2"])
def test_double_pair_passes_on_tensor_cores_folded_terms(oracle, monkeypatch, variant):
    """The tensor-core passes with XOR terms folded before and after the blocks (permutations
    inside the 16 x 16 tile matrix), random register."""
    monkeypatch.setenv("QGPU_PAIR2_TC", variant)
    n = 13
    rng = np.random.default_rng(77)
    reg = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    reg /= np.linalg.norm(reg)
    b = ProgramBuilder(n)
    for layer in range(8):
        for w in range(n):
            b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(layer % 2, n - 1, 2):
            b.add("CNot", w + 1, (w,))
        for w in range(n):
            b.add("Rx", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(1 - layer % 2, n - 1, 2):
            b.add("CNot", w + 1, (w,))
    prog = b.build()
    ref = oracle.simulate(prog, reg, engine=oracle.DENSE)
    out = run_gpu(prog, "fast", reg=reg)
    assert np.max(np.abs(out - ref)) <= TOL_FAST


@pytest.mark.parametrize("precision", [nat.QGPU_C128, nat.QGPU_C64])
@pytest.mark.parametrize("n", [8, 13])
def test_double_pair_passes_folded_xor_terms(oracle, precision, n):
    """Pair blocks two per pass (k_pair2) with the XOR layers between them folded in as tile
    permutations before and after the blocks: CNots across neighbouring blocks, CNots inside a
    block's wires, swaps across two blocks, and a Toffoli spanning two tiles (left in an XOR
    pass); random register, so every slot of a tile carries a distinct value."""
    rng = np.random.default_rng(40 + n)
    reg = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    reg /= np.linalg.norm(reg)
    b = ProgramBuilder(n)
    for layer in range(6):
        for w in range(n):
            b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(0, n - 1, 2):
            b.add("CNot", w + 1, (w,))
        for w in range(n):
            b.add("Rx", w, (), param=float(rng.uniform(0, 6.3)))
        if layer % 2 == 0:
            for w in range(1, n - 2, 2):
                b.add("CNot", w + 1, (w,))
            b.add("Toffoli", 7, (0, 3))
        else:
            b.add("Swap", 2, (5,))
            b.add("CNot", 1, (0,))
            b.add("CNot", 4, (3,))
            b.add("CNot", 7, (6,))
    prog = b.build()
    if precision == nat.QGPU_C64:
        reg = reg.astype(np.complex64).astype(np.complex128)
    ref = oracle.simulate(prog, reg, engine=oracle.DENSE)
    out = run_gpu(prog, "fast", precision=precision, reg=reg)
    tol = TOL_FAST if precision == nat.QGPU_C128 else 1e-5
    assert np.max(np.abs(out - ref)) <= tol


@pytest.mark.parametrize("precision", [nat.QGPU_C128, nat.QGPU_C64])
@pytest.mark.parametrize("n,pairs", [
    (12, [(i, 11 - i) for i in range(6)]),          # full bit reversal, even width
    (13, [(i, 12 - i) for i in range(6)]),          # odd width: middle wire stays
    (11, [(0, 5), (2, 9), (1, 10), (7, 3)]),        # scattered disjoint swaps
    (9, [(8, 7), (0, 1)]),                          # two swaps, all in the lowest tile bits
])
def test_swap_runs_bit_permutation(oracle, precision, n, pairs):
    """A run of disjoint Swap gates is one index-bit permutation (k_bitperm: tiles closed under
    the permutation, moved in pairs); random register, every wire distinct."""
    rng = np.random.default_rng(31 + n)
    reg = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    reg /= np.linalg.norm(reg)
    b = ProgramBuilder(n)
    for a, c in pairs:
        b.add("Swap", a, (c,))
    prog = b.build()
    if precision == nat.QGPU_C64:  # the register as the complex64 handle holds it
        reg = reg.astype(np.complex64).astype(np.complex128)
    ref = oracle.simulate(prog, reg, engine=oracle.DENSE)
    out = run_gpu(prog, "fast", precision=precision, reg=reg)
    assert np.array_equal(out, ref)  # a permutation moves values unchanged


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_custom_blocks_dense_nonunitary_and_wide(oracle, mode):
    """Custom gates: a dense 3-wire block with None entries, a non-unitary block, and the widest
    block (QGPU_MAX_OP_WIRES = 10 wires) on a register with an unused wire."""
    n = 11
    rng = np.random.default_rng(3)
    b = ProgramBuilder(n)
    for w in range(n):
        b.add("H", w)
    blk = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    b.add_custom(4, [9, 1], blk, np.array([0, 1, 0, 0, 1, 0, 0, 0], np.uint8))
    b.add_custom(2, [], np.array([[2 ** 0.5, 0], [0, 0]], np.complex128), np.zeros(2, np.uint8))
    d = 1 << 10
    wide = np.eye(d, dtype=np.complex128)[rng.permutation(d)] * np.exp(1j * rng.random(d))[:, None]
    b.add_custom(0, [10, 1, 2, 3, 4, 5, 6, 7, 8], wide, np.zeros(d, np.uint8))
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    out = run_gpu(prog, mode)
    if mode == "exact":
        assert np.array_equal(out, ref)
    else:
        assert np.max(np.abs(out - ref)) <= TOL_FAST * max(1.0, np.max(np.abs(ref)))


def test_complex64_consistency(oracle):
    prog = W.brickwork_qft(n=14, layers=20, seed=3)
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    out = run_gpu(prog, "fast", precision=nat.QGPU_C64)
    fid = abs(np.vdot(ref, out)) ** 2 / (np.vdot(out, out).real * np.vdot(ref, ref).real)
    assert 1.0 - fid <= 1e-8
    assert np.max(np.abs(out - ref)) <= 1e-5


def test_upload_download_roundtrip_and_reductions():
    rng = np.random.default_rng(1)
    n = 13
    a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    h = nat.Handle(n)
    h.upload(a)
    assert np.array_equal(h.download(), a)
    assert h.norm() == pytest.approx(float(np.sum(np.abs(a) ** 2)), rel=1e-13)
    assert h.checksum() == pytest.approx(complex(np.sum(a)), rel=1e-12, abs=1e-9)
    h.set_zero()
    z = h.download()
    assert z[0] == 1 and np.count_nonzero(z) == 1
    h64 = nat.Handle(n, nat.QGPU_C64)
    h64.upload(a)
    assert np.max(np.abs(h64.download() - a.astype(np.complex64))) == 0.0


def test_argument_errors_are_reported():
    h = nat.Handle(4)
    b = ProgramBuilder(4)
    b.add("CNot", 2, (2,))          # control equals target
    with pytest.raises(QuantrError):
        p = b.build()
        h.apply(p.ops, p.mats, p.none)
    b = ProgramBuilder(4)
    b.add("H", 4)                   # wire out of range
    with pytest.raises(QuantrError):
        p = b.build()
        h.apply(p.ops, p.mats, p.none)
    with pytest.raises(QuantrError):
        h.upload(np.zeros(8, np.complex128))  # wrong register size
    with pytest.raises(QuantrError):
        nat.Handle(40)               # 16 TiB of complex128: out of memory, reported
    empty = ProgramBuilder(4).build()
    h.apply(empty.ops, empty.mats, empty.none)  # empty program is a no-op
    assert h.download()[0] == 1


def test_single_qubit_register(oracle):
    b = ProgramBuilder(1)
    for name in ("H", "T", "Y", "Rx", "S"):
        b.add(name, 0, (), param=0.9)
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    assert np.array_equal(run_gpu(prog, "exact"), ref)
    assert np.max(np.abs(run_gpu(prog, "fast") - ref)) <= TOL_FAST


# ---------------------------------------------------------------------------------------------
# measurement
# ---------------------------------------------------------------------------------------------
def _near_boundary(state, u, tol=1e-12):
    cum = np.cumsum(np.abs(state) ** 2)
    j = np.searchsorted(cum, u, side="right")
    lo = np.abs(u - cum[np.clip(j - 1, 0, cum.size - 1)])
    hi = np.abs(u - cum[np.clip(j, 0, cum.size - 1)])
    return np.minimum(lo, hi) < tol


@pytest.mark.parametrize("n", [3, 7, 12, 16])
def test_shot_rule_matches_linear_scan(oracle, n):
    prog = W.random_columns(n=n, columns=10, seed=n)
    state = oracle.simulate(prog, engine=oracle.DENSE)
    h = nat.Handle(n)
    h.upload(state)
    rng = np.random.default_rng(n)
    u = rng.random(20000)
    u[:3] = [0.0, np.nextafter(1.0, 0.0), 0.5]
    got = h.measure_uniforms(u)
    want = oracle.measure_uniforms(state, u)
    differ = got != want
    assert not np.any(differ & ~_near_boundary(state, u))


def test_shots_none_beyond_total_probability(oracle):
    n = 5
    state = np.full(1 << n, (0.5 / (1 << n)) ** 0.5, dtype=np.complex128)  # total 0.5
    h = nat.Handle(n)
    h.upload(state)
    u = np.array([0.1, 0.49, 0.51, 0.9])
    assert np.array_equal(h.measure_uniforms(u), oracle.measure_uniforms(state, u))
    idx, cnt, failed = h.measure(10000, seed=3)
    assert 4000 < failed < 6000 and cnt.sum() + failed == 10000


def test_measure_all_chi_square(oracle):
    scipy_stats = pytest.importorskip("scipy.stats")
    prog = W.random_columns(n=12, seed=1)
    state = oracle.simulate(prog, engine=oracle.DENSE)
    h = nat.Handle(12)
    h.upload(state)
    shots = 200000
    idx, cnt, failed = h.measure(shots, seed=1234)
    assert failed == 0 and cnt.sum() == shots and np.all(np.diff(idx.astype(np.int64)) > 0)
    obs = np.zeros(1 << 12)
    obs[idx.astype(np.int64)] = cnt
    exp = np.abs(state) ** 2 * shots
    order = np.argsort(exp)
    # merge the smallest bins until each merged bin expects >= 5
    o_m, e_m, acc_o, acc_e = [], [], 0.0, 0.0
    for i in order:
        acc_o += obs[i]
        acc_e += exp[i]
        if acc_e >= 5:
            o_m.append(acc_o)
            e_m.append(acc_e)
            acc_o = acc_e = 0.0
    if acc_e > 0:
        o_m[-1] += acc_o
        e_m[-1] += acc_e
    o_m, e_m = np.array(o_m), np.array(e_m)
    chi2 = float(np.sum((o_m - e_m) ** 2 / e_m))
    p = scipy_stats.chi2.sf(chi2, len(o_m) - 1)
    assert p > 1e-4, (chi2, len(o_m))


def test_grovers_histogram_thresholds():
    """tests/grovers.rs:62-69: measure_all(500) finds only 011 and 111, each > 200 times."""
    sim = G.grovers_3qubit_circuit().simulate()
    bins = sim.measure_all(500).take()
    for state, count in bins.items():
        if str(state) in ("011", "111"):
            assert count > 200
        else:
            assert count == 0


def test_x3sudoko_histogram_thresholds():
    """tests/grovers.rs:141-152: measure_all(5000) on the 10-qubit sudoku oracle."""
    sim = G.x3sudoko_circuit().simulate()
    sim.print_warnings(True)
    bins = sim.measure_all(5000).take()
    for state, count in bins.items():
        if str(state)[:6] in G.X3SUDOKO_SOLUTIONS:
            assert count > 150
        else:
            assert count < 150


def test_measure_all_without_cache_post_select():
    """examples/post_select.rs with per-shot re-simulation: every shot sees |x0x> outcomes."""
    qc = Circuit(3)
    qc.add_repeating_gate(Gate.H, [0, 1, 2]).add_gate(Gate.Custom(G.post_select, [], "P"), 1)
    sim = qc.simulate()
    sim.print_warnings(True)
    bins = sim.measure_all_without_cache(20).take()
    assert sum(bins.values()) == 20
    assert all(str(s)[1] == "0" for s in bins)


def _launches_of_one_simulate(qc):
    sim = qc.clone_and_simulate()
    return sim.handle.launch_count()


def test_measure_all_without_cache_deterministic_simulates_once():
    """Identical tables for every shot: shots 2..N come from one re-simulation from |0...0>,
    sampled in one call; the histogram follows |a|^2 of the |0...0> run."""
    n = 10
    qc = W.brickwork_qft_circuit(n, layers=3, seed=41)

    def custom_x(ps):  # deterministic, unitary
        out = ps.comp_basis() ^ 1
        return SuperPosition.new_with_amplitudes([1.0 if i == out else 0.0 for i in range(2)])

    qc.add_gate(Gate.Custom(custom_x, [], "X"), 1)
    per_sim = _launches_of_one_simulate(qc)
    sim = qc.clone_and_simulate()
    sim.print_warnings(True)
    probs = np.abs(sim.get_state().take().get_amplitudes()) ** 2
    before = sim.handle.launch_count()
    shots = 20000
    bins = sim.measure_all_without_cache(shots).take()
    used = sim.handle.launch_count() - before
    assert sum(bins.values()) == shots
    assert used <= 2 * per_sim + 64, (used, per_sim)
    counts = np.zeros(2**n)
    for s, c in bins.items():
        counts[s.comp_basis()] += c
    exp = probs / probs.sum() * shots
    m = exp >= 5
    chi2 = float((((counts - exp) ** 2)[m] / exp[m]).sum())
    assert chi2 < m.sum() + 6 * math.sqrt(2 * m.sum()) + 60


def test_measure_all_without_cache_stochastic_custom_redraws():
    """A Custom function that draws a bit-flip per call (a mixed-state channel): each shot
    re-tabulates it, so the outcome frequency follows the flip probability."""
    draw = np.random.default_rng(7)
    p = 0.3

    def flip(ps):
        bit = 1 if draw.random() < p else 0
        out = ps.comp_basis() ^ bit
        return SuperPosition.new_with_amplitudes([1.0 if i == out else 0.0 for i in range(2)])

    qc = Circuit(1)
    qc.add_gate(Gate.Custom(flip, [], "F"), 0)
    sim = qc.simulate()
    sim.print_warnings(True)
    shots = 3000
    bins = sim.measure_all_without_cache(shots).take()
    ones = sum(c for s, c in bins.items() if str(s) == "1")
    assert sum(bins.values()) == shots
    sd = math.sqrt(shots * p * (1 - p))
    assert abs(ones - shots * p) < 6 * sd + 1


def test_fast_mode_keeps_range_of_growing_custom_blocks(oracle):
    """Custom gates that scale a wire by 2^60, applied twice (amplitudes up to ~2^120): beyond the
    float pairs' exponent range, so the fast mode runs the program with native f64 arithmetic
    (the plan's growth bound) and stays within 1e-12 relative of the oracle instead of
    overflowing."""
    n = 9
    b = ProgramBuilder(n)
    for w in range(n):
        b.add("H", w)
        b.add("Ry", w, (), param=0.1 * (w + 1))
    big = np.array([[2.0 ** 60, 0], [0, 2.0 ** 60]], np.complex128)
    b.add_custom(3, [], big, np.zeros(2, np.uint8))
    b.add("CNot", 4, (3,))
    b.add_custom(5, [], big, np.zeros(2, np.uint8))
    for w in range(n):
        b.add("Rz", w, (), param=0.2 * w)
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    out = run_gpu(prog, "fast")
    assert np.all(np.isfinite(out))
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))

