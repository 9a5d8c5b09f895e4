// quantr.hpp — header-only C++ mirror of quantr's public API (crate 0.6.0, src/lib.rs:78-84) over
// the C ABI of libquantr_gpu (qgpu.h). Simulation runs on the GPU; there is no CPU fallback.
//
//   quantr::Circuit qc = quantr::Circuit::new_(3);
//   qc.add_gate(quantr::Gate::H(), 2).add_gate(quantr::Gate::CNot(2), 1);
//   quantr::SimulatedCircuit sim = std::move(qc).simulate();
//   auto amps = sim.get_state().take().get_amplitudes();
//   auto bins = sim.measure_all(500).take();           // std::map<ProductState, size_t>
//
// Names, argument meaning and error messages follow the Rust crate; Rust's `Result::Err` becomes
// a thrown quantr::QuantrError. Link with -lquantr_gpu.
#pragma once

#include <algorithm>
#include <charconv>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdint>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "qgpu.h"

namespace quantr {

using Complex64 = std::complex<double>;

// src/error.rs:17-33
struct QuantrError : std::runtime_error {
    std::string message;
    explicit QuantrError(const std::string& m)
        : std::runtime_error("\x1b[91m[Quantr Error] " + m + "\x1b[0m "), message(m) {}
};

inline void check(int status) {
    if (status != QGPU_OK) throw QuantrError(qgpu_last_error());
}

inline uint64_t& shot_seed() {
    static uint64_t s = 0;
    return s;
}
// `fastrand::seed` counterpart: reseeds the stream that keys each measure_all call and the draws
// of SuperPosition::measure.
inline void seed(uint64_t s) { shot_seed() = s; }
// one uniform double in [0, 1) from the shot stream: the stream steps (64-bit LCG) and its state
// goes through the SplitMix64 finaliser; (x >> 11) 2^-53
inline double next_shot_uniform() {
    uint64_t z = shot_seed() = shot_seed() * 6364136223846793005ull + 1442695040888963407ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// an f64 as Rust's `{}` prints it: the fewest digits that read back to the same value, never an
// exponent (2.0 -> "2", 1e-7 -> "0.0000001")
inline std::string rust_f64(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    char buf[400];
    const auto r = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::fixed);
    return std::string(buf, r.ptr);
}
// an f64 as Rust's `{:?}` prints it: like `{}` with at least one fractional digit, but in
// exponent form (no '+', no leading zeros: "1e-5", "1.5e16") below 1e-4 and from 1e16
inline std::string rust_f64_debug(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    const double a = std::fabs(x);
    if (a == 0 || (a >= 1e-4 && a < 1e16)) {
        std::string s = rust_f64(x);
        if (s.find('.') == std::string::npos) s += ".0";
        return s;
    }
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::scientific);
    const std::string s(buf, r.ptr);  // shortest digits, e.g. "1e-05", "1.5e+16"
    const size_t e = s.find('e');
    return s.substr(0, e) + "e" + std::to_string(std::stoi(s.substr(e + 1)));
}
// a string as Rust's `{:?}` prints it: quoted, with \\, \", \n, \r, \t, \0 and other control
// characters escaped
inline std::string rust_str_debug(const std::string& v) {
    std::string o = "\"";
    for (unsigned char c : v) {
        switch (c) {
            case '\\': o += "\\\\"; break;
            case '"': o += "\\\""; break;
            case '\n': o += "\\n"; break;
            case '\r': o += "\\r"; break;
            case '\t': o += "\\t"; break;
            case '\0': o += "\\0"; break;
            default:
                if (c < 0x20 || c == 0x7f) {
                    char b[16];
                    std::snprintf(b, sizeof b, "\\u{%x}", c);
                    o += b;
                } else {
                    o += (char)c;
                }
        }
    }
    return o + "\"";
}

// ---- states (src/circuit/states/) -----------------------------------------------------------
enum class Qubit : uint8_t { Zero = 0, One = 1 };

class ProductState {
   public:
    std::vector<Qubit> qubits;

    ProductState() = default;
    explicit ProductState(std::vector<Qubit> q) : qubits(std::move(q)) {}
    static ProductState new_(const std::vector<Qubit>& q) {  // product_states.rs:37-48
        if (q.empty())
            throw QuantrError("The slice of qubits is empty, it needs to at least have one element.");
        return ProductState(q);
    }
    static ProductState binary_basis(uint64_t index, size_t n) {  // product_states.rs:205-215
        std::vector<Qubit> q(n);
        for (size_t w = 0; w < n; ++w) q[w] = ((index >> (n - 1 - w)) & 1u) ? Qubit::One : Qubit::Zero;
        return ProductState(q);
    }
    uint64_t comp_basis() const {  // product_states.rs:191-201 (64-bit)
        uint64_t v = 0;
        for (Qubit q : qubits) v = (v << 1) | (uint64_t)q;
        return v;
    }
    const Qubit* get(size_t i) const { return i < qubits.size() ? &qubits[i] : nullptr; }
    const std::vector<Qubit>& get_qubits() const { return qubits; }
    std::vector<Qubit>& get_mut_qubits() { return qubits; }
    size_t num_qubits() const { return qubits.size(); }
    ProductState& invert_digit(size_t place) {
        if (place >= qubits.size())
            throw QuantrError("The position of the binary digit, " + std::to_string(place) +
                              ", is out of bounds. The product dimension is " +
                              std::to_string(qubits.size()) +
                              ", and so the position must be strictly less.");
        qubits[place] = qubits[place] == Qubit::Zero ? Qubit::One : Qubit::Zero;
        return *this;
    }
    ProductState kronecker_prod(Qubit q) const {  // product_states.rs:180-183
        ProductState p = *this;
        p.qubits.push_back(q);
        return p;
    }
    static ProductState from(Qubit q) { return ProductState({q}); }  // From<Qubit>
    // the qubits in order (product_states_iter.rs)
    std::vector<Qubit>::const_iterator begin() const { return qubits.begin(); }
    std::vector<Qubit>::const_iterator end() const { return qubits.end(); }
    std::string to_string() const {
        std::string s;
        for (Qubit q : qubits) s += q == Qubit::One ? '1' : '0';
        return s;
    }
    bool operator==(const ProductState& o) const { return qubits == o.qubits; }
    bool operator!=(const ProductState& o) const { return qubits != o.qubits; }
    bool operator<(const ProductState& o) const { return qubits < o.qubits; }
};

// Qubit::kronecker_prod (qubit.rs:35-37): |a> (x) |b> = |ab>
inline ProductState kronecker_prod(Qubit a, Qubit b) { return ProductState({a, b}); }

class SuperPosition {
    // |num - cmp| < 1e-6 (super_positions.rs:18, 246-248)
    static bool equal_within_error(double num, double cmp) {
        return num < cmp + 1e-6 && num > cmp - 1e-6;
    }
    static double norm_sqr_sum(const std::vector<Complex64>& a) {  // sequential, like `.sum()`
        double t = 0;
        for (const Complex64& x : a) t += x.real() * x.real() + x.imag() * x.imag();
        return t;
    }
    static size_t trailing_zeros(size_t len) {  // usize::trailing_zeros (64 for 0)
        size_t n = 0;
        if (len == 0) return 8 * sizeof(size_t);
        while (!((len >> n) & 1u)) ++n;
        return n;
    }

   public:
    std::vector<Complex64> amplitudes;
    size_t product_dim = 0;

    SuperPosition() = default;
    SuperPosition(std::vector<Complex64> a, size_t n) : amplitudes(std::move(a)), product_dim(n) {}
    static SuperPosition new_(size_t n) {
        if (n == 0) throw QuantrError("The number of qubits must be non-zero.");
        std::vector<Complex64> a((size_t)1 << n);
        a[0] = 1.0;
        return SuperPosition(std::move(a), n);
    }
    static SuperPosition new_with_amplitudes(const std::vector<Complex64>& a) {  // super_positions.rs:68-91
        if (!equal_within_error(norm_sqr_sum(a), 1.0))
            throw QuantrError("Slice given to set amplitudes in super position does not conserve "
                              "probability, the absolute square sum of the coefficents must be one.");
        const size_t len = a.size();
        if (len == 0 || (len & (len - 1)))
            throw QuantrError("The length of the array must be of the form 2**n where n is an integer.");
        return SuperPosition(a, trailing_zeros(len));
    }
    // super_positions_unchecked.rs:64-70: no checks; the product dimension is the length's
    // trailing zero count
    static SuperPosition new_with_amplitudes_unchecked(const std::vector<Complex64>& a) {
        return SuperPosition(a, trailing_zeros(a.size()));
    }
    // super_positions.rs:105-131: states missing from the map have amplitude zero
    static SuperPosition new_with_hash_amplitudes(const std::map<ProductState, Complex64>& h) {
        if (h.empty())
            throw QuantrError("An empty HashMap was given. A superposition must have at least one "
                              "non-zero state.");
        const size_t dim = h.begin()->first.num_qubits();
        double total = 0;
        for (const auto& [st, amp] : h) {
            if (st.num_qubits() != dim)
                throw QuantrError("The first state has product dimension of " + std::to_string(dim) +
                                  ", whilst the state, |" + st.to_string() +
                                  ">, found as a key in the HashMap has dimension " +
                                  std::to_string(st.num_qubits()) + ".");
            total += amp.real() * amp.real() + amp.imag() * amp.imag();
        }
        if (!equal_within_error(total, 1.0))
            throw QuantrError("The total sum of the absolute square of all amplitudes, " +
                              rust_f64(total) +
                              ", does not equal 1. That is, the superpositon does not conserve "
                              "probability.");
        std::vector<Complex64> a((size_t)1 << dim);
        for (const auto& [st, amp] : h) a[st.comp_basis()] = amp;
        return SuperPosition(std::move(a), dim);
    }
    static SuperPosition from(const ProductState& p) {
        std::vector<Complex64> a((size_t)1 << p.num_qubits());
        a[p.comp_basis()] = 1.0;
        return SuperPosition(std::move(a), p.num_qubits());
    }
    static SuperPosition from(Qubit q) { return from(ProductState::from(q)); }
    std::optional<Complex64> get_amplitude(size_t i) const {
        if (i < amplitudes.size()) return amplitudes[i];
        return std::nullopt;
    }
    size_t get_num_qubits() const { return product_dim; }
    size_t get_dimension() const { return amplitudes.size(); }
    const std::vector<Complex64>& get_amplitudes() const { return amplitudes; }
    Complex64 get_amplitude_from_state(const ProductState& p) const {
        if (((size_t)1 << p.num_qubits()) != amplitudes.size())
            throw QuantrError("Unable to retreive product state, |\"" + p.to_string() +
                              "\"> with dimension " + std::to_string(p.num_qubits()) +
                              ". The superposition is a linear combination of states with "
                              "different dimension. These dimensions should be equal.");
        return amplitudes[p.comp_basis()];
    }
    SuperPosition& set_amplitudes(const std::vector<Complex64>& a) {  // super_positions.rs:229-244
        if (a.size() != amplitudes.size())
            throw QuantrError("The slice given to set the amplitudes in the computational basis has "
                              "length " + std::to_string(a.size()) + ", when it should have length " +
                              std::to_string(amplitudes.size()) + ".");
        if (!equal_within_error(norm_sqr_sum(a), 1.0))
            throw QuantrError("Slice given to set amplitudes in super position does not conserve "
                              "probability, the absolute square sum of the coefficents must be one.");
        amplitudes = a;
        return *this;
    }
    // super_positions_unchecked.rs:74-77: no checks, the product dimension is left as it was
    SuperPosition& set_amplitudes_unchecked(const std::vector<Complex64>& a) {
        amplitudes = a;
        return *this;
    }
    // super_positions.rs:270-299: every state of the register takes its amplitude from the map,
    // or zero
    SuperPosition& set_amplitudes_from_states(const std::map<ProductState, Complex64>& h) {
        if (h.empty())
            throw QuantrError("An empty HashMap was given. A superposition must have at least one "
                              "non-zero state.");
        const size_t dim = trailing_zeros(amplitudes.size());
        double total = 0;
        for (const auto& [st, amp] : h) {
            if (st.num_qubits() != dim)
                throw QuantrError("The first state has product dimension of " + std::to_string(dim) +
                                  ", whilst the state, |" + st.to_string() +
                                  ">, found as a key in the HashMap has dimension " +
                                  std::to_string(st.num_qubits()) + ".");
            total += amp.real() * amp.real() + amp.imag() * amp.imag();
        }
        if (!equal_within_error(total, 1.0))
            throw QuantrError("The total sum of the absolute square of all amplitudes does not equal "
                              "1. That is, the superpositon does not conserve probability.");
        std::fill(amplitudes.begin(), amplitudes.end(), Complex64(0.0, 0.0));
        for (const auto& [st, amp] : h) amplitudes[st.comp_basis()] = amp;
        return *this;
    }
    std::map<ProductState, Complex64> to_hash_map() const {  // super_positions.rs:315-323
        std::map<ProductState, Complex64> m;
        for (size_t i = 0; i < amplitudes.size(); ++i) {
            const double p = amplitudes[i].real() * amplitudes[i].real() +
                             amplitudes[i].imag() * amplitudes[i].imag();
            if (!equal_within_error(p, 0.0)) m[ProductState::binary_basis(i, product_dim)] = amplitudes[i];
        }
        return m;
    }
    // One shot of the host-side container (super_positions.rs:332-342): the first state whose
    // running sum of |a_i|^2 exceeds u, or nothing when u reaches the total (a register left
    // unnormalised by a non-unitary Custom gate). `measure()` draws u from the shot stream
    // (quantr draws it with `fastrand::f64()`); registers on the device are sampled by
    // SimulatedCircuit::measure_all.
    std::optional<ProductState> measure_with(double u) const {
        double cum = 0;
        for (size_t i = 0; i < amplitudes.size(); ++i) {
            cum += amplitudes[i].real() * amplitudes[i].real() + amplitudes[i].imag() * amplitudes[i].imag();
            if (u < cum) return ProductState::binary_basis(i, product_dim);
        }
        return std::nullopt;
    }
    std::optional<ProductState> measure() const { return measure_with(next_shot_uniform()); }
    // `for (auto [state, amp] : superpos)` (super_position_iter.rs:19-47): every basis state in
    // index order with its amplitude
    struct Iter {
        const SuperPosition* sp;
        size_t i;
        std::pair<ProductState, Complex64> operator*() const {
            return {ProductState::binary_basis(i, sp->product_dim), sp->amplitudes[i]};
        }
        Iter& operator++() {
            ++i;
            return *this;
        }
        bool operator!=(const Iter& o) const { return i != o.i; }
    };
    Iter begin() const { return {this, 0}; }
    Iter end() const { return {this, amplitudes.size()}; }
    // #[derive(PartialEq)] (super_positions.rs:21): amplitudes and product dimension
    bool operator==(const SuperPosition& o) const {
        return product_dim == o.product_dim && amplitudes == o.amplitudes;
    }
    bool operator!=(const SuperPosition& o) const { return !(*this == o); }
};

// ---- gates (src/circuit/gate.rs:19-106) --------------------------------------------------------
using CustomFn = std::function<std::optional<SuperPosition>(const ProductState&)>;

struct Gate {
    int kind = QGPU_GATE_ID;
    double angle = 0.0;
    int k = 0;
    std::vector<size_t> controls;
    CustomFn func;
    std::string name;
    const void* func_id = nullptr;  // identity of the Custom function for equality

    static Gate make(int kind, std::vector<size_t> c = {}, double a = 0.0, int k = 0) {
        Gate g;
        g.kind = kind;
        g.controls = std::move(c);
        g.angle = a;
        g.k = k;
        return g;
    }
    static Gate Id() { return make(QGPU_GATE_ID); }
    static Gate H() { return make(QGPU_GATE_H); }
    static Gate X() { return make(QGPU_GATE_X); }
    static Gate Y() { return make(QGPU_GATE_Y); }
    static Gate Z() { return make(QGPU_GATE_Z); }
    static Gate S() { return make(QGPU_GATE_S); }
    static Gate Sdag() { return make(QGPU_GATE_SDAG); }
    static Gate T() { return make(QGPU_GATE_T); }
    static Gate Tdag() { return make(QGPU_GATE_TDAG); }
    static Gate X90() { return make(QGPU_GATE_X90); }
    static Gate Y90() { return make(QGPU_GATE_Y90); }
    static Gate MX90() { return make(QGPU_GATE_MX90); }
    static Gate MY90() { return make(QGPU_GATE_MY90); }
    static Gate Rx(double a) { return make(QGPU_GATE_RX, {}, a); }
    static Gate Ry(double a) { return make(QGPU_GATE_RY, {}, a); }
    static Gate Rz(double a) { return make(QGPU_GATE_RZ, {}, a); }
    static Gate Phase(double a) { return make(QGPU_GATE_PHASE, {}, a); }
    static Gate CR(double a, size_t c) { return make(QGPU_GATE_CR, {c}, a); }
    static Gate CRk(int kk, size_t c) { return make(QGPU_GATE_CRK, {c}, 0.0, kk); }
    static Gate CZ(size_t c) { return make(QGPU_GATE_CZ, {c}); }
    static Gate CY(size_t c) { return make(QGPU_GATE_CY, {c}); }
    static Gate CNot(size_t c) { return make(QGPU_GATE_CNOT, {c}); }
    static Gate Swap(size_t c) { return make(QGPU_GATE_SWAP, {c}); }
    static Gate Toffoli(size_t c1, size_t c2) { return make(QGPU_GATE_TOFFOLI, {c1, c2}); }
    static Gate Custom(std::optional<SuperPosition> (*f)(const ProductState&),
                       std::vector<size_t> c, std::string nm) {
        Gate g = make(QGPU_GATE_CUSTOM, std::move(c));
        g.func = f;
        g.func_id = (const void*)f;
        g.name = std::move(nm);
        return g;
    }
    bool is_single_gate() const { return kind >= QGPU_GATE_ID && kind <= QGPU_GATE_PHASE; }
    bool is_custom_gate() const { return kind == QGPU_GATE_CUSTOM; }
    std::optional<std::vector<size_t>> get_nodes() const {
        if (is_single_gate()) return std::nullopt;
        return controls;
    }
    bool operator==(const Gate& o) const {
        return kind == o.kind && angle == o.angle && k == o.k && controls == o.controls &&
               func_id == o.func_id && name == o.name;
    }
    bool operator!=(const Gate& o) const { return !(*this == o); }
    // `{:?}` of the Rust enum (the `#[derive(Debug)]` of gate.rs:18), as quantr's validation
    // messages print it: "H", "Rx(0.5)", "CRk(3, 1)", "Toffoli(0, 2)"; a Custom gate's function
    // pointer prints as its address
    std::string debug() const {
        static const char* const names[] = {
            "Id", "H", "X", "Y", "Z", "S", "Sdag", "T", "Tdag", "Rx", "Ry", "Rz", "X90", "Y90",
            "MX90", "MY90", "Phase", "CR", "CRk", "CZ", "CY", "CNot", "Swap", "Toffoli", "Custom"};
        const std::string nm = kind >= 0 && kind < QGPU_GATE_COUNT ? names[kind] : "?";
        auto list = [](const std::vector<size_t>& v) {
            std::string o = "[";
            for (size_t i = 0; i < v.size(); ++i) o += (i ? ", " : "") + std::to_string(v[i]);
            return o + "]";
        };
        switch (kind) {
            case QGPU_GATE_RX: case QGPU_GATE_RY: case QGPU_GATE_RZ: case QGPU_GATE_PHASE:
                return nm + "(" + rust_f64_debug(angle) + ")";
            case QGPU_GATE_CR:
                return nm + "(" + rust_f64_debug(angle) + ", " + std::to_string(controls[0]) + ")";
            case QGPU_GATE_CRK:
                return nm + "(" + std::to_string(k) + ", " + std::to_string(controls[0]) + ")";
            case QGPU_GATE_CZ: case QGPU_GATE_CY: case QGPU_GATE_CNOT: case QGPU_GATE_SWAP:
                return nm + "(" + std::to_string(controls[0]) + ")";
            case QGPU_GATE_TOFFOLI:
                return nm + "(" + std::to_string(controls[0]) + ", " + std::to_string(controls[1]) + ")";
            case QGPU_GATE_CUSTOM: {
                char a[32];
                std::snprintf(a, sizeof a, "%p", func_id);
                return nm + "(" + a + ", " + list(controls) + ", " + rust_str_debug(name) + ")";
            }
            default:
                return nm;
        }
    }
};

template <class T>
struct Measurement {  // src/circuit/measurement.rs:16-27
    bool observable;
    T value;
    T take() { return std::move(value); }
};

// ---- simulation result (src/simulated_circuit.rs) ----------------------------------------------
struct HandleDeleter {
    void operator()(qgpu_handle* h) const { qgpu_destroy(h); }
};
using Handle = std::unique_ptr<qgpu_handle, HandleDeleter>;

// The flat gate list as a gate program (simulation.rs:37-56): `Id` skipped, wire = index % n,
// every Custom tabulated by calling its function on each local basis state
// (simulation.rs:137-156).
struct Program {
    std::vector<qgpu_op> ops;
    std::vector<double> mats;
    std::vector<uint8_t> none;
};

inline Program lower(const std::vector<Gate>& gates, size_t n, bool progress) {
    Program p;
    size_t counter = 0;
    if (progress) std::cout << "Starting circuit simulation...\n";  // simulation.rs:32-34
    for (const Gate& g : gates) {
        if (g.kind == QGPU_GATE_ID) {
            ++counter;
            continue;
        }
        qgpu_op op{};
        op.kind = g.kind;
        op.target = (int32_t)(counter % n);
        op.n_controls = (int32_t)g.controls.size();
        for (size_t m = 0; m < g.controls.size() && m < QGPU_MAX_OP_WIRES; ++m)
            op.controls[m] = (int32_t)g.controls[m];
        op.param = g.angle;
        op.k = g.k;
        if (g.is_custom_gate()) {
            const size_t kq = g.controls.size() + 1, d = (size_t)1 << kq;
            op.mat_offset = (int64_t)p.mats.size();
            op.none_offset = (int64_t)p.none.size();
            for (size_t j = 0; j < d; ++j) {
                auto img = g.func(ProductState::binary_basis(j, kq));
                p.none.push_back(img ? 0 : 1);
                for (size_t l = 0; l < d; ++l) {
                    Complex64 v = (img && l < img->amplitudes.size()) ? img->amplitudes[l] : 0.0;
                    p.mats.push_back(v.real());
                    p.mats.push_back(v.imag());
                }
            }
        }
        if (progress) {  // simulation.rs:183-200
            std::cout << "Applying " << g.debug() << " on wire " << op.target << " # "
                      << counter + 1 << "/" << gates.size() << " \n";
            if (counter + 1 == gates.size()) std::cout << "Finished circuit simulation.\n";
        }
        p.ops.push_back(op);
        ++counter;
    }
    return p;
}

inline void apply(qgpu_handle* h, const Program& p) {
    check(qgpu_apply_program(h, p.ops.data(), p.ops.size(), p.mats.data(), p.mats.size(),
                             p.none.data(), p.none.size()));
}

class SimulatedCircuit {
   public:
    SimulatedCircuit(std::vector<Gate> g, size_t n, Handle h, bool progress)
        : circuit_gates_(std::move(g)), num_qubits_(n), handle_(std::move(h)), progress_(progress) {}

    Measurement<std::map<ProductState, size_t>> measure_all(size_t shots) const {
        if (!disable_warnings_)
            for (const Gate& g : circuit_gates_)
                if (g.is_custom_gate()) {
                    std::cerr << "\x1b[93m[Quantr Warning] Custom gates were detected in the "
                                 "circuit. Measurements will be taken from a cached register in "
                                 "memory, and so if the Custom gate does NOT implement a unitary "
                                 "mapping, the measure_all method will most likely lead to wrong "
                                 "results. To simulate a circuit without cache, see "
                                 "SimulatedCircuit::measure_all_without_cache.\x1b[0m\n";
                    break;
                }
        const size_t cap = std::min<size_t>(shots, (size_t)1 << std::min<size_t>(num_qubits_, 40));
        std::vector<uint64_t> idx(cap ? cap : 1), cnt(cap ? cap : 1);
        size_t nu = 0;
        uint64_t failed = 0;
        shot_seed() = shot_seed() * 6364136223846793005ull + 1442695040888963407ull;
        check(qgpu_measure(handle_.get(), shots, shot_seed(), idx.data(), cnt.data(), cap, &nu,
                           &failed));
        std::map<ProductState, size_t> bins;
        for (size_t i = 0; i < nu; ++i)
            bins[ProductState::binary_basis(idx[i], num_qubits_)] = (size_t)cnt[i];
        if (!disable_warnings_)  // once per failed shot (add_to_bin, simulated_circuit.rs:116-130)
            for (uint64_t f = 0; f < failed; ++f)
                std::cerr << "\x1b[93m[Quantr Warning] The superposition failed to collapse to a "
                             "state during repeat measurements. This is likely due to the use of "
                             "Gate::Custom where the mapping is not unitary.\x1b[0m\n";
        return {true, std::move(bins)};
    }
    // simulated_circuit.rs:81-114. Shot 1 from the cached register, later shots from a
    // re-simulation from |0...0> with every Custom re-tabulated (a function drawing random Kraus
    // branches gets a fresh draw per shot). Consecutive shots whose tables are identical share one
    // re-simulation and one sampler call.
    Measurement<std::map<ProductState, size_t>> measure_all_without_cache(size_t shots) {
        if (shots == 0) throw QuantrError("measure_all_without_cache needs at least one shot.");
        std::map<ProductState, size_t> bins;
        auto add = [&](size_t count) {
            const size_t cap = std::min<size_t>(count, (size_t)1 << std::min<size_t>(num_qubits_, 40));
            std::vector<uint64_t> idx(cap ? cap : 1), cnt(cap ? cap : 1);
            size_t nu = 0;
            uint64_t failed = 0;
            shot_seed() = shot_seed() * 6364136223846793005ull + 1442695040888963407ull;
            check(qgpu_measure(handle_.get(), count, shot_seed(), idx.data(), cnt.data(), cap, &nu,
                               &failed));
            for (size_t i = 0; i < nu; ++i)
                bins[ProductState::binary_basis(idx[i], num_qubits_)] += (size_t)cnt[i];
            if (!disable_warnings_)
                for (uint64_t f = 0; f < failed; ++f)
                    std::cerr << "\x1b[93m[Quantr Warning] The superposition failed to collapse to "
                                 "a state during repeat measurements. This is likely due to the "
                                 "use of Gate::Custom where the mapping is not unitary.\x1b[0m\n";
        };
        add(1);
        if (progress_) std::cout << "Measured state # 1/" << shots << "\n";
        bool stochastic = false;
        for (const Gate& g : circuit_gates_) stochastic |= g.is_custom_gate();
        std::optional<Program> last;
        size_t pending = 0;
        for (size_t s = 0; s + 1 < shots; ++s) {
            if (!last || stochastic) {
                Program p = lower(circuit_gates_, num_qubits_, progress_);
                if (!last || p.mats != last->mats || p.none != last->none) {
                    if (pending) add(pending);
                    pending = 0;
                    check(qgpu_set_zero(handle_.get()));
                    apply(handle_.get(), p);
                    last = std::move(p);
                }
            }
            ++pending;
            if (progress_)
                std::cout << "Register reset to zero state\nMeasured state # " << s + 2 << "/"
                          << shots << "\n";
        }
        if (pending) add(pending);
        return {true, std::move(bins)};
    }
    Measurement<SuperPosition> get_state() const {
        std::vector<Complex64> a((size_t)1 << num_qubits_);
        check(qgpu_download(handle_.get(), reinterpret_cast<double*>(a.data()), a.size()));
        return {false, SuperPosition(std::move(a), num_qubits_)};
    }
    Measurement<SuperPosition> take_state() const { return get_state(); }
    // get_state().take().to_hash_map() computed on the device: only survivors are copied back.
    std::map<ProductState, Complex64> state_hash_map(double margin = 1e-6) const {
        size_t n = 0;
        int st = qgpu_extract_nonzero(handle_.get(), margin, nullptr, nullptr, 0, &n);
        if (st != QGPU_OK && st != QGPU_ERR_INVALID) check(st);
        std::vector<uint64_t> idx(n ? n : 1);
        std::vector<Complex64> amp(n ? n : 1);
        check(qgpu_extract_nonzero(handle_.get(), margin, idx.data(),
                                   reinterpret_cast<double*>(amp.data()), n, &n));
        std::map<ProductState, Complex64> m;
        for (size_t i = 0; i < n; ++i) m[ProductState::binary_basis(idx[i], num_qubits_)] = amp[i];
        return m;
    }
    void print_warnings(bool printing) { disable_warnings_ = printing; }
    const std::vector<Gate>& get_circuit_gates() const { return circuit_gates_; }
    size_t get_num_qubits() const { return num_qubits_; }
    void set_print_progress(bool p) { progress_ = p; }
    qgpu_handle* handle() const { return handle_.get(); }

   private:
    std::vector<Gate> circuit_gates_;
    size_t num_qubits_;
    Handle handle_;
    bool progress_;
    bool disable_warnings_ = false;
};

// ---- circuit (src/circuit.rs) -------------------------------------------------------------------
class Circuit {
   public:
    static Circuit new_(size_t n) {  // circuit.rs:48-62
        if (n == 0) throw QuantrError("The initialised circuit must have at least one wire.");
        Circuit c;
        c.num_qubits_ = n;
        return c;
    }
    size_t get_num_qubits() const { return num_qubits_; }
    void set_print_progress(bool p) { progress_ = p; }
    const std::vector<Gate>& get_gates() const { return gates_; }
    // Engine options (not in quantr): QGPU_C128/QGPU_C64 and QGPU_MODE_*.
    Circuit& set_backend(int precision, int mode) {
        precision_ = precision;
        mode_ = mode;
        return *this;
    }

    Circuit& add_gate(const Gate& g, size_t position) { return add_gates_with_positions({{position, g}}); }

    Circuit& add_gates_with_positions(const std::map<size_t, Gate>& gp) {  // circuit.rs:152-188
        for (auto& kv : gp)
            if (kv.first >= num_qubits_)
                throw QuantrError("The position, " + std::to_string(kv.first) +
                                  ", is out of bounds for the circuit with " +
                                  std::to_string(num_qubits_) + " qubits.");
        std::vector<Gate> col(num_qubits_, Gate::Id());
        for (auto& kv : gp) col[kv.first] = kv.second;
        overlapping(col);
        push_multi_gates(col);
        gates_.insert(gates_.end(), col.begin(), col.end());
        return *this;
    }

    Circuit& add_gates(const std::vector<Gate>& gates) {  // circuit.rs:210-226
        if (gates.size() != num_qubits_)
            throw QuantrError("The number of gates, " + std::to_string(gates.size()) +
                              ", does not match the number of wires, " +
                              std::to_string(num_qubits_) + ". All wires must have gates added.");
        std::vector<Gate> col = gates;
        overlapping(col);
        push_multi_gates(col);
        gates_.insert(gates_.end(), col.begin(), col.end());
        return *this;
    }

    // circuit.rs:324-341. A position beyond the register gets the out-of-bounds message of
    // add_gates_with_positions (quantr's repeat scan indexes past its table and panics there).
    Circuit& add_repeating_gate(const Gate& g, const std::vector<size_t>& pos) {
        std::vector<bool> seen(num_qubits_, false);
        bool repeated = false;
        for (size_t p : pos) {
            if (p >= num_qubits_)
                throw QuantrError("The position, " + std::to_string(p) +
                                  ", is out of bounds for the circuit with " +
                                  std::to_string(num_qubits_) + " qubits.");
            repeated = repeated || seen[p];
            seen[p] = true;
        }
        if (repeated) {
            std::string list = "[";
            for (size_t i = 0; i < pos.size(); ++i) list += (i ? ", " : "") + std::to_string(pos[i]);
            throw QuantrError("Attempted to add more than one gate onto a single wire. The positions "
                              "in " + list + "] must all differ.");
        }
        std::vector<Gate> col(num_qubits_, Gate::Id());
        for (size_t p : pos) col[p] = g;
        return add_gates(col);
    }

    Circuit& change_register(const SuperPosition& s) {  // circuit.rs:463-473
        if (s.product_dim != num_qubits_)
            throw QuantrError("The custom register has a product state dimension of " +
                              std::to_string(s.product_dim) + ", while the number of qubits is " +
                              std::to_string(num_qubits_) + ". These must equal each other.");
        register_ = s;
        return *this;
    }

    SimulatedCircuit simulate() && {  // circuit.rs:364-388
        auto reg = std::move(register_);
        register_.reset();
        return run(reg);
    }
    SimulatedCircuit clone_and_simulate() const { return run(register_); }

   private:
    std::vector<Gate> gates_;
    size_t num_qubits_ = 0;
    std::optional<SuperPosition> register_;
    bool progress_ = false;
    int precision_ = QGPU_C128;
    int mode_ = QGPU_MODE_FAST;

    static void push_multi_gates(std::vector<Gate>& gates) {  // circuit.rs:230-270
        bool found_multi = false, found_second = false;
        for (const Gate& g : gates) {
            if (g.is_custom_gate())
                for (unsigned char ch : g.name)
                    if (ch > 127)
                        throw QuantrError("The custom function name, " + g.name +
                                          ", does not only use ASCII chars. This could lead to "
                                          "problems in printing the circuit diagram. This warning "
                                          "will be promoted to an Error in the next major release.");
            if (g != Gate::Id()) {
                if (found_multi) {
                    found_second = true;
                    break;
                }
                found_multi = true;
            }
        }
        if (!found_second) return;
        std::vector<Gate> extended;
        for (size_t pos = 0; pos < gates.size(); ++pos)
            if (!gates[pos].is_single_gate()) {
                std::vector<Gate> col(gates.size(), Gate::Id());
                col[pos] = gates[pos];
                extended.insert(extended.end(), col.begin(), col.end());
                gates[pos] = Gate::Id();
            }
        gates.insert(gates.end(), extended.begin(), extended.end());
    }

    // circuit.rs:272-293, in its order: repeated nodes, then a node on the gate's own wire. A
    // node beyond the register is reported first with the crate's message for it (quantr's own
    // repeat scan indexes past its table there and panics before reaching that message).
    void overlapping(const std::vector<Gate>& gates) const {
        for (size_t pos = 0; pos < gates.size(); ++pos) {
            auto nodes = gates[pos].get_nodes();
            if (!nodes) continue;
            for (size_t nd : *nodes)
                if (nd >= num_qubits_)
                    throw QuantrError("The control node at position " + std::to_string(nd) +
                                      ", is greater than the umnber of qubits " +
                                      std::to_string(num_qubits_) + ".");
            std::vector<bool> seen(num_qubits_, false);
            for (size_t nd : *nodes) {
                if (seen[nd])
                    throw QuantrError("The gate, " + gates[pos].debug() +
                                      ", has overlapping control nodes.");
                seen[nd] = true;
            }
            for (size_t nd : *nodes)
                if (nd == pos)
                    throw QuantrError("The gate, " + gates[pos].debug() +
                                      ", has a control node that equals the gate's position " +
                                      std::to_string(pos) + ".");
        }
    }

    SimulatedCircuit run(const std::optional<SuperPosition>& reg) const {
        qgpu_handle* raw = nullptr;
        check(qgpu_create((int)num_qubits_, precision_, &raw));
        Handle h(raw);
        check(qgpu_set_mode(h.get(), mode_));
        if (reg)
            check(qgpu_upload(h.get(), reinterpret_cast<const double*>(reg->amplitudes.data()),
                              reg->amplitudes.size()));
        apply(h.get(), lower(gates_, num_qubits_, progress_));  // simulation.rs:37-56
        return SimulatedCircuit(gates_, num_qubits_, std::move(h), progress_);
    }
};

}  // namespace quantr

// #[derive(Hash)] on ProductState (product_states.rs:18): usable as an unordered_map key, as
// quantr uses it in its HashMaps
namespace std {
template <>
struct hash<quantr::ProductState> {
    size_t operator()(const quantr::ProductState& p) const noexcept {
        uint64_t x = 0xcbf29ce484222325ull ^ (uint64_t)p.qubits.size();  // FNV-1a over the qubits
        for (quantr::Qubit q : p.qubits) x = (x ^ (uint64_t)q) * 0x100000001b3ull;
        return (size_t)x;
    }
};
}  // namespace std
