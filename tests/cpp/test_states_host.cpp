// test_states_host.cpp — the host-side parts of include/quantr.hpp: the state containers
// (ProductState, SuperPosition, Qubit) against the cases of quantr's own unit tests and doc
// examples (src/circuit/states/super_positions.rs:396-545, product_states.rs:274-330 and the doc
// comments of both files), gate formatting and circuit validation messages (circuit.rs:272-293).
// None of these makes a library call, so the program needs neither the library nor a GPU.
// Prints "<n> failure(s)".
#include <cmath>
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <unordered_map>

#include "quantr.hpp"

using quantr::Complex64;
using quantr::ProductState;
using quantr::Qubit;
using quantr::QuantrError;
using quantr::SuperPosition;

static int failures = 0;
#define CHECK(cond)                                                   \
    do {                                                              \
        if (!(cond)) {                                                \
            ++failures;                                               \
            std::printf("FAIL line %d: %s\n", __LINE__, #cond);       \
        }                                                             \
    } while (0)

// runs f, which must throw QuantrError; returns its message ("" when nothing was thrown)
template <class F>
static std::string error_of(F f) {
    try {
        f();
    } catch (const QuantrError& e) {
        return e.message;
    }
    return "";
}

static bool starts_with(const std::string& s, const std::string& p) { return s.rfind(p, 0) == 0; }

int main() {
    const double r = M_SQRT1_2;
    const Complex64 z(0, 0), re(r, 0), im(0, -r);
    const ProductState s01({Qubit::Zero, Qubit::One}), s10({Qubit::One, Qubit::Zero});

    // retrieve_amplitude_from_state / retrieve_amplitude_from_list_pos
    SuperPosition sp = SuperPosition::new_(2);
    sp.set_amplitudes({z, re, im, z});
    CHECK(sp.get_amplitude_from_state(s01) == re);
    CHECK(sp.get_amplitude(2).value() == im);
    // catches_retrieve_amplitude_from_wrong_list_pos: `None`
    CHECK(!sp.get_amplitude(4).has_value());
    // catches_retrieve_amplitude_from_wrong_state
    CHECK(starts_with(error_of([&] { sp.get_amplitude_from_state(ProductState({Qubit::Zero, Qubit::One, Qubit::One})); }),
                      "Unable to retreive product state, |\"011\"> with dimension 3."));
    // catches_super_position_breaking_conservation
    CHECK(starts_with(error_of([&] { SuperPosition::new_(2).set_amplitudes({z, {0.5, 0}, z, {0, -0.5}}); }),
                      "Slice given to set amplitudes in super position does not conserve probability"));
    CHECK(error_of([&] { SuperPosition::new_(2).set_amplitudes({z, re}); }) ==
          "The slice given to set the amplitudes in the computational basis has length 2, when it "
          "should have length 4.");

    // sets_amplitude_from_states
    const std::map<ProductState, Complex64> states{{s01, re}, {s10, im}};
    CHECK(SuperPosition::new_with_hash_amplitudes(states).amplitudes ==
          SuperPosition::new_with_amplitudes({z, re, im, z}).amplitudes);
    CHECK(SuperPosition::new_with_hash_amplitudes(states).get_num_qubits() == 2);
    // sets_amplitude_from_states_wrong_dimension (the first key of the ordered map is |01>)
    const ProductState s101({Qubit::One, Qubit::Zero, Qubit::One});
    CHECK(error_of([&] { SuperPosition::new_with_hash_amplitudes({{s01, re}, {s101, im}}); }) ==
          "The first state has product dimension of 2, whilst the state, |101>, found as a key in "
          "the HashMap has dimension 3.");
    // sets_amplitude_from_states_breaks_probability: the total printed as Rust prints an f64
    const std::string eb = error_of([&] { SuperPosition::new_with_hash_amplitudes({{s01, re}, {s10, im * 0.5}}); });
    CHECK(starts_with(eb, "The total sum of the absolute square of all amplitudes, 0.625"));
    CHECK(eb.find(", does not equal 1. That is, the superpositon does not conserve probability.") !=
          std::string::npos);
    CHECK(error_of([&] { SuperPosition::new_with_hash_amplitudes({}); }) ==
          "An empty HashMap was given. A superposition must have at least one non-zero state.");

    // doc examples: new_with_hash_amplitudes, set_amplitudes_from_states, to_hash_map
    CHECK(SuperPosition::new_with_hash_amplitudes({{s01, {1, 0}}}).amplitudes ==
          std::vector<Complex64>({z, {1, 0}, z, z}));
    SuperPosition sq = SuperPosition::new_(2);
    sq.set_amplitudes_from_states({{s01, {1, 0}}});
    CHECK(sq.amplitudes == std::vector<Complex64>({z, {1, 0}, z, z}));  // |00> zeroed
    CHECK(starts_with(error_of([&] { sq.set_amplitudes_from_states({{s01, {0.5, 0}}}); }),
                      "The total sum of the absolute square of all amplitudes does not equal 1."));
    CHECK(starts_with(error_of([&] { sq.set_amplitudes_from_states({{s101, {1, 0}}}); }),
                      "The first state has product dimension of 2, whilst the state, |101>"));
    const auto hm = SuperPosition::new_(2).to_hash_map();
    CHECK(hm.size() == 1 && hm.count(ProductState({Qubit::Zero, Qubit::Zero})) == 1);
    CHECK(sp.to_hash_map().size() == 2);

    // unchecked forms: no checks, product dimension = trailing zeros of the length
    CHECK(SuperPosition::new_with_amplitudes_unchecked(std::vector<Complex64>(6)).get_num_qubits() == 1);
    CHECK(SuperPosition::new_with_amplitudes_unchecked(std::vector<Complex64>(8)).get_num_qubits() == 3);
    SuperPosition su = SuperPosition::new_(1);
    su.set_amplitudes_unchecked({{2, 0}, {0, 3}});
    CHECK(su.amplitudes[1] == Complex64(0, 3) && su.get_num_qubits() == 1);
    CHECK(starts_with(error_of([] { SuperPosition::new_with_amplitudes({{0.6, 0}, {0.8, 0}, {0, 0}}); }),
                      "The length of the array must be of the form 2**n"));

    // measure: the first i with u < cumulative |a_i|^2 (0.36 and 0.64 here), else nothing
    const SuperPosition m = SuperPosition::new_with_amplitudes({{0.6, 0}, {0, 0.8}});
    CHECK(m.measure_with(0.0).value().to_string() == "0");
    CHECK(m.measure_with(0.3599).value().to_string() == "0");
    CHECK(m.measure_with(0.3601).value().to_string() == "1");
    CHECK(m.measure_with(0.9999).value().to_string() == "1");
    const SuperPosition half = SuperPosition::new_with_amplitudes_unchecked({{0.5, 0}, {0.5, 0}});
    CHECK(!half.measure_with(0.6).has_value());  // total 0.5: the shot fails
    quantr::seed(0);
    int ones = 0;
    const int shots = 20000;
    for (int i = 0; i < shots; ++i) ones += m.measure().value().to_string() == "1";
    CHECK(std::fabs((double)ones / shots - 0.64) < 0.02);
    quantr::seed(0);
    int ones2 = 0;
    for (int i = 0; i < shots; ++i) ones2 += m.measure().value().to_string() == "1";
    CHECK(ones == ones2);  // reseeding repeats the stream

    // equality (derived PartialEq): amplitudes and dimension
    CHECK(SuperPosition::new_with_hash_amplitudes(states) == SuperPosition::new_with_amplitudes({z, re, im, z}));
    CHECK(SuperPosition::new_(2) != SuperPosition::new_with_amplitudes({z, re, im, z}));
    CHECK(s01 != s10);
    std::unordered_map<ProductState, int> hashed{{s01, 1}, {s10, 2}};  // derived Hash
    CHECK(hashed.at(ProductState({Qubit::Zero, Qubit::One})) == 1 && hashed.size() == 2);
    CHECK(std::hash<ProductState>()(s01) != std::hash<ProductState>()(s10));

    // iteration over a superposition: (state, amplitude) in index order
    std::string seen;
    for (auto [st, a] : sp) seen += st.to_string() + (a == z ? "z " : "a ");
    CHECK(seen == "00z 01a 10a 11z ");

    // ProductState: iterates_through_qubits, converts_from_integer_to_product_state,
    // inverting_binary_digit, Display, kronecker products, From<Qubit>
    std::string q;
    for (Qubit x : ProductState::new_({Qubit::One, Qubit::Zero, Qubit::One})) q += x == Qubit::One ? '1' : '0';
    CHECK(q == "101");
    CHECK(ProductState::binary_basis(6, 3) == ProductState({Qubit::One, Qubit::One, Qubit::Zero}));
    ProductState inv({Qubit::One, Qubit::One, Qubit::Zero});
    inv.invert_digit(2);
    CHECK(inv == ProductState({Qubit::One, Qubit::One, Qubit::One}));
    CHECK(starts_with(error_of([&] { inv.invert_digit(3); }), "The position of the binary digit, 3, is out of bounds."));
    CHECK(s01.to_string() == "01");
    CHECK(quantr::kronecker_prod(Qubit::Zero, Qubit::One) == s01);
    CHECK(ProductState::new_({Qubit::Zero, Qubit::Zero}).kronecker_prod(Qubit::One).to_string() == "001");
    CHECK(ProductState::from(Qubit::One).get_qubits() == std::vector<Qubit>({Qubit::One}));
    CHECK(SuperPosition::from(Qubit::One).amplitudes == std::vector<Complex64>({z, {1, 0}}));
    CHECK(error_of([] { ProductState::new_({}); }) ==
          "The slice of qubits is empty, it needs to at least have one element.");

    // f64 in messages as Rust's `{}` prints it
    CHECK(quantr::rust_f64(2.0) == "2");
    CHECK(quantr::rust_f64(0.5) == "0.5");
    CHECK(quantr::rust_f64(1e-7) == "0.0000001");
    CHECK(quantr::rust_f64(0.1 + 0.2) == "0.30000000000000004");
    CHECK(quantr::rust_f64(-0.0) == "-0");
    CHECK(quantr::rust_f64(1e21) == "1000000000000000000000");

    CHECK(quantr::rust_f64_debug(1.0) == "1.0");
    CHECK(quantr::rust_f64_debug(0.5) == "0.5");
    CHECK(quantr::rust_f64_debug(1e-5) == "1e-5");
    CHECK(quantr::rust_f64_debug(-2.5e-7) == "-2.5e-7");
    CHECK(quantr::rust_f64_debug(1e16) == "1e16");
    CHECK(quantr::rust_f64_debug(1234.5) == "1234.5");
    CHECK(quantr::rust_str_debug("a\"b\\c\n") == "\"a\\\"b\\\\c\\n\"");

    // gates as the crate's messages print them (`{:?}` of the enum)
    using quantr::Circuit;
    using quantr::Gate;
    CHECK(Gate::H().debug() == "H");
    CHECK(Gate::Rx(0.5).debug() == "Rx(0.5)");
    CHECK(Gate::Phase(1.0).debug() == "Phase(1.0)");
    CHECK(Gate::Rz(1e-5).debug() == "Rz(1e-5)");
    CHECK(Gate::CR(2.0, 1).debug() == "CR(2.0, 1)");
    CHECK(Gate::CRk(3, 1).debug() == "CRk(3, 1)");
    CHECK(Gate::CNot(2).debug() == "CNot(2)");
    CHECK(Gate::Toffoli(0, 2).debug() == "Toffoli(0, 2)");
    const std::string cd = Gate::Custom([](const ProductState&) -> std::optional<SuperPosition> { return std::nullopt; },
                                        {0, 1}, "q\"x").debug();
    CHECK(starts_with(cd, "Custom(0x") && cd.size() > 20 &&
          cd.substr(cd.size() - 17) == ", [0, 1], \"q\\\"x\")");

    // circuit.rs:272-293 messages and their order: repeated nodes before a node on the gate's
    // own wire; a node beyond the register (quantr panics in its repeat scan there)
    CHECK(error_of([] { Circuit::new_(3).add_gates({Gate::CNot(0), Gate::Id(), Gate::Id()}); }) ==
          "The gate, CNot(0), has a control node that equals the gate's position 0.");
    CHECK(error_of([] { Circuit::new_(3).add_gates({Gate::Toffoli(0, 0), Gate::Id(), Gate::Id()}); }) ==
          "The gate, Toffoli(0, 0), has overlapping control nodes.");
    CHECK(error_of([] { Circuit::new_(3).add_gates_with_positions({{2, Gate::H()}, {0, Gate::CNot(2)}, {1, Gate::CNot(3)}}); }) ==
          "The control node at position 3, is greater than the umnber of qubits 3.");
    CHECK(error_of([] { Circuit::new_(3).add_gates({Gate::CNot(1), Gate::Id(), Gate::Id()}); }).empty());
    auto fn = [](const ProductState&) -> std::optional<SuperPosition> { return std::nullopt; };
    CHECK(error_of([&] { Circuit::new_(3).add_gate(Gate::Custom(fn, {0}, "NonAscii\xe2\x80\xa0"), 1); }) ==
          "The custom function name, NonAscii\xe2\x80\xa0, does not only use ASCII chars. This could "
          "lead to problems in printing the circuit diagram. This warning will be promoted to an "
          "Error in the next major release.");
    CHECK(error_of([] { Circuit::new_(2).add_gates({Gate::H()}); }) ==
          "The number of gates, 1, does not match the number of wires, 2. All wires must have gates added.");
    CHECK(error_of([] { Circuit::new_(2).add_gate(Gate::H(), 2); }) ==
          "The position, 2, is out of bounds for the circuit with 2 qubits.");
    CHECK(error_of([] { Circuit::new_(0); }) == "The initialised circuit must have at least one wire.");
    CHECK(error_of([] { Circuit::new_(4).add_repeating_gate(Gate::X(), {0, 1, 1, 3}); }) ==
          "Attempted to add more than one gate onto a single wire. The positions in [0, 1, 1, 3] "
          "must all differ.");
    CHECK(error_of([] { Circuit::new_(3).add_repeating_gate(Gate::H(), {0, 3}); }) ==
          "The position, 3, is out of bounds for the circuit with 3 qubits.");
    CHECK(Circuit::new_(3).add_repeating_gate(Gate::H(), {2, 0}).get_gates().size() == 3);

    // set_print_progress output while lowering (simulation.rs:32-34, 183-200): Id skipped, the
    // gate printed with `{:?}`, the counter over every gate of the flat list
    {
        std::ostringstream log;
        std::streambuf* old = std::cout.rdbuf(log.rdbuf());
        quantr::lower({Gate::H(), Gate::Id(), Gate::CNot(0), Gate::Id(), Gate::Rz(0.5), Gate::Id()}, 3, true);
        quantr::lower({Gate::Id(), Gate::X()}, 2, true);
        std::cout.rdbuf(old);
        CHECK(log.str() ==
              "Starting circuit simulation...\n"
              "Applying H on wire 0 # 1/6 \n"
              "Applying CNot(0) on wire 2 # 3/6 \n"
              "Applying Rz(0.5) on wire 1 # 5/6 \n"
              "Starting circuit simulation...\n"
              "Applying X on wire 1 # 2/2 \n"
              "Finished circuit simulation.\n");
    }

    std::printf("%d failure(s)\n", failures);
    return failures != 0;
}
