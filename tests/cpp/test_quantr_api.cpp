// The quantr crate's own test cases, written against the C++ mirror (include/quantr.hpp) and run
// on the GPU engine. Exit code 0 when every case passes; one line per case on stdout.
#include <cmath>
#include <cstdio>
#include <string>

#include "quantr.hpp"

using quantr::Circuit;
using quantr::Complex64;
using quantr::Gate;
using quantr::ProductState;
using quantr::Qubit;
using quantr::SuperPosition;

static int failures = 0;
static const double R = 0.70710678118654752440;

static void expect_state(const char* name, Circuit qc, const std::vector<Complex64>& want,
                         double tol) {
    auto sim = std::move(qc).simulate();
    auto got = sim.get_state().take().get_amplitudes();
    double err = 0;
    for (size_t i = 0; i < want.size(); ++i) err = std::max(err, std::abs(got[i] - want[i]));
    const bool ok = got.size() == want.size() && err < tol;
    std::printf("%s %s (max err %.2e)\n", ok ? "PASS" : "FAIL", name, err);
    if (!ok) ++failures;
}

static std::vector<Complex64> amps(size_t n, std::map<size_t, Complex64> e) {
    std::vector<Complex64> a((size_t)1 << n);
    for (auto& kv : e) a[kv.first] = kv.second;
    return a;
}

// src/circuit.rs:504-512
static std::optional<SuperPosition> example_cnot(const ProductState& p) {
    const auto& q = p.get_qubits();
    if (q[0] == Qubit::Zero) return std::nullopt;
    if (q[1] == Qubit::Zero) return SuperPosition::new_with_amplitudes({0, 0, 0, 1});
    return SuperPosition::new_with_amplitudes({0, 0, 1, 0});
}

// tests/qft.rs:51-67: a Custom gate that simulates a nested circuit
static std::optional<SuperPosition> qft(const ProductState& in) {
    const size_t n = in.num_qubits();
    Circuit mini = Circuit::new_(n);
    for (size_t pos = 0; pos < n; ++pos) {
        mini.add_gate(Gate::H(), pos);
        for (size_t k = 2; k <= n - pos; ++k) mini.add_gate(Gate::CRk((int)k, pos + k - 1), pos);
    }
    mini.change_register(SuperPosition::from(in));
    return std::move(mini).simulate().take_state().take();
}

template <class F>
static void expect_error(const char* name, F f) {
    bool thrown = false;
    try {
        f();
    } catch (const quantr::QuantrError&) {
        thrown = true;
    }
    std::printf("%s %s\n", thrown ? "PASS" : "FAIL", name);
    if (!thrown) ++failures;
}

int main() {
    {  // src/circuit.rs:604-613
        Circuit c = Circuit::new_(2);
        c.add_gates({Gate::H(), Gate::H()}).add_gates({Gate::S(), Gate::Sdag()});
        expect_state("swap_and_conjugate_gates", std::move(c),
                     amps(2, {{0, 0.5}, {1, Complex64(0, -0.5)}, {2, Complex64(0, 0.5)}, {3, 0.5}}), 1e-6);
    }
    {  // :629-641
        Circuit c = Circuit::new_(3);
        c.add_gate(Gate::H(), 2).add_gate(Gate::Custom(example_cnot, {2}, "cNot"), 1);
        expect_state("custom_gates", std::move(c), amps(3, {{0, R}, {3, R}}), 1e-6);
    }
    {  // :644-658
        Circuit c = Circuit::new_(4);
        c.add_gate(Gate::X(), 0).add_gate(Gate::H(), 3).add_gate(Gate::Y(), 3).add_gate(Gate::Toffoli(3, 0), 1);
        expect_state("toffoli_gates", std::move(c), amps(4, {{8, Complex64(0, -R)}, {13, Complex64(0, R)}}), 1e-6);
    }
    {  // :751-768
        Circuit c = Circuit::new_(4);
        c.add_repeating_gate(Gate::X(), {1, 2}).add_gate(Gate::CY(2), 0).add_gate(Gate::Swap(3), 2)
            .add_gate(Gate::CY(0), 3);
        expect_state("cy_and_swap_gates_work", std::move(c), amps(4, {{12, 1.0}}), 1e-6);
    }
    {  // :940-952
        Circuit c = Circuit::new_(3);
        c.add_gates({Gate::X(), Gate::X(), Gate::X()}).add_gate(Gate::CR(-M_PI * 0.5, 2), 1);
        expect_state("cr_gate", std::move(c), amps(3, {{7, Complex64(0, -1)}}), 1e-6);
    }
    {  // :970-982
        Circuit c = Circuit::new_(3);
        c.add_gate(Gate::X(), 1).change_register(
            SuperPosition::from(ProductState({Qubit::One, Qubit::Zero, Qubit::One})));
        expect_state("custom_register", std::move(c), amps(3, {{7, 1.0}}), 1e-6);
    }
    {  // tests/qft.rs:21-47
        Circuit c = Circuit::new_(3);
        c.add_repeating_gate(Gate::X(), {1, 2}).add_gate(Gate::Custom(qft, {0, 1}, "QFT"), 2);
        expect_state("simple_qft", std::move(c),
                     amps(3, {{0, R * 0.5}, {1, -R * 0.5}, {2, Complex64(0, -R * 0.5)},
                              {3, Complex64(0, R * 0.5)}, {4, Complex64(-0.25, 0.25)},
                              {5, Complex64(0.25, -0.25)}, {6, Complex64(0.25, 0.25)},
                              {7, Complex64(-0.25, -0.25)}}), 1e-8);
    }
    {  // tests/grovers.rs:21-72, including the measure_all(500) thresholds
        Circuit c = Circuit::new_(3);
        c.add_repeating_gate(Gate::H(), {0, 1, 2}).add_gate(Gate::CZ(1), 2)
            .add_repeating_gate(Gate::H(), {0, 1, 2}).add_repeating_gate(Gate::X(), {0, 1, 2})
            .add_gate(Gate::H(), 2).add_gate(Gate::Toffoli(0, 1), 2).add_gate(Gate::H(), 2)
            .add_repeating_gate(Gate::X(), {0, 1, 2}).add_repeating_gate(Gate::H(), {0, 1, 2});
        quantr::seed(0);
        auto sim = std::move(c).simulate();
        auto bins = sim.measure_all(500).take();
        bool ok = true;
        for (auto& kv : bins) {
            const std::string s = kv.first.to_string();
            if (s == "011" || s == "111") ok = ok && kv.second > 200;
            else ok = ok && kv.second == 0;
        }
        std::printf("%s grovers_3qubit_histogram\n", ok ? "PASS" : "FAIL");
        if (!ok) ++failures;
    }
    {  // src/circuit.rs:535-550: the pushed column layout
        Circuit c = Circuit::new_(3);
        c.add_gates({Gate::CNot(2), Gate::CNot(0), Gate::H()})
            .add_gates({Gate::Toffoli(1, 2), Gate::H(), Gate::CNot(0)});
        std::vector<Gate> want = {Gate::Id(), Gate::Id(), Gate::H(), Gate::CNot(2), Gate::Id(), Gate::Id(),
                                  Gate::Id(), Gate::CNot(0), Gate::Id(), Gate::Id(), Gate::H(), Gate::Id(),
                                  Gate::Toffoli(1, 2), Gate::Id(), Gate::Id(), Gate::Id(), Gate::Id(),
                                  Gate::CNot(0)};
        const bool ok = c.get_gates() == want;
        std::printf("%s pushes_multi_gates\n", ok ? "PASS" : "FAIL");
        if (!ok) ++failures;
    }
    {  // device-side to_hash_map equals the host rule on the downloaded register
        Circuit c = Circuit::new_(10);
        c.add_gate(Gate::H(), 0);
        for (size_t t = 1; t < 10; ++t) c.add_gate(Gate::CNot(0), t);
        c.add_gate(Gate::Ry(0.7), 4);
        auto sim = std::move(c).simulate();
        auto dev = sim.state_hash_map();
        auto host = sim.get_state().take().to_hash_map();
        const bool ok = dev == host && dev.size() == 4;
        std::printf("%s state_hash_map\n", ok ? "PASS" : "FAIL");
        if (!ok) ++failures;
    }
    {  // simulated_circuit.rs:81-114 on a uniform 3-qubit register: every bin near shots/8
        Circuit c = Circuit::new_(3);
        c.add_repeating_gate(Gate::H(), {0, 1, 2});
        auto sim = std::move(c).simulate();
        auto bins = sim.measure_all_without_cache(4000).take();
        size_t total = 0;
        bool ok = bins.size() == 8;
        for (auto& kv : bins) {
            total += kv.second;
            ok = ok && kv.second > 350 && kv.second < 650;
        }
        ok = ok && total == 4000;
        std::printf("%s measure_all_without_cache\n", ok ? "PASS" : "FAIL");
        if (!ok) ++failures;
    }
    expect_error("catches_overlapping_control_nodes",
                 [] { Circuit::new_(3).add_gates({Gate::CNot(0), Gate::Id(), Gate::Id()}); });
    expect_error("control_node_greater_than_circuit_size",
                 [] { Circuit::new_(3).add_gates_with_positions({{2, Gate::H()}, {0, Gate::CNot(2)}, {1, Gate::CNot(3)}}); });
    expect_error("custom_register_wrong_dimension", [] {
        Circuit::new_(3).add_gate(Gate::X(), 1).change_register(
            SuperPosition::from(ProductState({Qubit::One, Qubit::Zero})));
    });
    std::printf("%d failure(s)\n", failures);
    return failures ? 1 : 0;
}
