// lower_dump.cpp — the C++ mirror's lowering (include/quantr.hpp: quantr::lower, the gate-program
// side of simulation.rs:37-56 and the Custom tabulation of simulation.rs:137-156) on a fixed
// circuit, written as the raw qgpu_op records, Custom block doubles and None flags for a byte
// comparison with the Python mirror's lowering. No library call; needs no GPU.
//
// usage: lower_dump ops.bin mats.bin none.bin
#include <cstdio>
#include <fstream>

#include "quantr.hpp"

using namespace quantr;

// examples/custom_gate.rs:46-62
static std::optional<SuperPosition> cccnot(const ProductState& p) {
    const auto& q = p.get_qubits();
    const std::vector<Qubit> a{Qubit::One, Qubit::One, Qubit::One, Qubit::Zero};
    const std::vector<Qubit> b{Qubit::One, Qubit::One, Qubit::One, Qubit::One};
    if (q == a) return SuperPosition::from(ProductState(b));
    if (q == b) return SuperPosition::from(ProductState(a));
    return std::nullopt;
}

// src/circuit.rs:504-512
static std::optional<SuperPosition> example_cnot(const ProductState& p) {
    const auto& q = p.get_qubits();
    if (q[0] == Qubit::Zero) return std::nullopt;
    if (q[1] == Qubit::Zero) return SuperPosition::new_with_amplitudes({0, 0, 0, 1});
    return SuperPosition::new_with_amplitudes({0, 0, 1, 0});
}

// a non-unitary one-wire map with a complex image (examples/post_select.rs style)
static std::optional<SuperPosition> scaled(const ProductState& p) {
    if (p.get_qubits()[0] == Qubit::Zero)
        return SuperPosition::new_with_amplitudes_unchecked({Complex64(0.6, 0.1), Complex64(0, -0.3)});
    return SuperPosition::new_with_amplitudes_unchecked({Complex64(0, 0), Complex64(0, 0)});
}

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    Circuit qc = Circuit::new_(5);
    qc.add_repeating_gate(Gate::H(), {0, 1, 2, 3, 4});
    qc.add_gates({Gate::X(), Gate::Y(), Gate::Z(), Gate::S(), Gate::Sdag()});
    qc.add_gates({Gate::T(), Gate::Tdag(), Gate::X90(), Gate::Y90(), Gate::MX90()});
    qc.add_gates({Gate::MY90(), Gate::Rx(0.25), Gate::Ry(-1.5), Gate::Rz(3.0), Gate::Phase(0.7)});
    qc.add_gate(Gate::CR(1.1, 0), 3).add_gate(Gate::CRk(3, 4), 1).add_gate(Gate::CZ(2), 0);
    qc.add_gate(Gate::CY(1), 4).add_gate(Gate::CNot(0), 2).add_gate(Gate::Swap(4), 1);
    qc.add_gate(Gate::Toffoli(0, 4), 2);
    qc.add_gate(Gate::Custom(cccnot, {0, 1, 2}, "X"), 3);
    qc.add_gate(Gate::Custom(example_cnot, {4}, "X"), 0);
    qc.add_gate(Gate::Custom(scaled, {}, "P"), 2);
    qc.add_gates({Gate::Id(), Gate::CNot(4), Gate::Id(), Gate::H(), Gate::Rx(0.5)});
    const Program p = lower(qc.get_gates(), qc.get_num_qubits(), false);
    std::ofstream(argv[1], std::ios::binary)
        .write(reinterpret_cast<const char*>(p.ops.data()), (std::streamsize)(p.ops.size() * sizeof(qgpu_op)));
    std::ofstream(argv[2], std::ios::binary)
        .write(reinterpret_cast<const char*>(p.mats.data()), (std::streamsize)(p.mats.size() * 8));
    std::ofstream(argv[3], std::ios::binary)
        .write(reinterpret_cast<const char*>(p.none.data()), (std::streamsize)p.none.size());
    std::printf("ops %zu mats %zu none %zu\n", p.ops.size(), p.mats.size(), p.none.size());
    return 0;
}
