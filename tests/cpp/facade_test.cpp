// Quaru's own tests (tests/register_operation_tests.rs, src/register.rs:437-445,
// examples/quantum_teleportation.rs, examples/openqasm_example.rs) written
// against the C++ facade include/quaru/quaru.hpp. Exit status 0 = all passed.
#include <cmath>
#include <cstdio>
#include <fstream>

#include "quaru/quaru.hpp"

using namespace quaru;
namespace op = quaru::operation;

static int failures = 0;
#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);    \
            failures++;                                                   \
        }                                                                 \
    } while (0)

static bool equal_qubits(const std::vector<c64>& a, const std::vector<c64>& b) {
    for (size_t i = 0; i < a.size(); i++)
        if (std::abs(a[i] - b[i]) >= 1e-8) return false;
    return true;
}

int main(int argc, char** argv) {
    const std::string tmp = argc > 1 ? argv[1] : "/tmp";
    {  // measure_on_zero_state_gives_false
        Register r = Register::new_({false});
        r.seed(1);
        CHECK(r.measure(0) == false);
    }
    {  // from_qubits_test
        const double s = 1.0 / std::sqrt(2.0);
        Register a = Register::from_qubits({{1.0, 0.0}, {0.0, 1.0}, {s, s}});
        Register b = Register::new_({false, true, false});
        b.apply(op::hadamard(2));
        CHECK(a == b);
    }
    for (size_t i = 0; i < 3; i++) {  // hadamard_hadamard_retains_original_state, test_not_on_arbitrary_qubit
        Register r = Register::new_({false, false, false});
        Register e = r.clone();
        r.apply(op::hadamard(i)).apply(op::hadamard(i));
        CHECK(r == e);
        r.apply(op::not_(i));
        CHECK(r.measure(i) == true);
    }
    for (size_t i = 0; i < 5; i++) {  // first_bell_state_measure_equal
        Register r = Register::new_(std::vector<bool>(6, false));
        r.seed(i);
        r.apply(op::hadamard(i)).apply(op::cnot(i, i + 1));
        CHECK(r.measure(i) == r.measure(i + 1));
    }
    for (size_t n = 2; n <= 6; n++)  // toffoli_test (all-ones inputs flip the target)
        for (int bits = 0; bits < 64; bits += 7) {
            std::vector<bool> init(6);
            for (int b = 0; b < 6; b++) init[b] = (bits >> b) & 1;
            Register r = Register::new_(init);
            std::vector<size_t> ctrl;
            for (size_t c = 0; c + 1 < n; c++) ctrl.push_back(c);
            r.apply(op::cnx(ctrl, n - 1));
            bool all = true;
            for (size_t c = 0; c + 1 < n; c++) all &= r.measure(c);
            const bool t = r.measure(n - 1);
            CHECK(all ? t != init[n - 1] : t == init[n - 1]);
        }
    for (size_t n = 2; n <= 6; n++) {  // apply_all_test
        Register a = Register::new_(std::vector<bool>(n, false)), b = Register::new_(std::vector<bool>(n, false));
        for (size_t i = 0; i < n; i++) a.apply(op::hadamard(i));
        b.apply_all(op::hadamard(0));
        CHECK(a == b);
        auto e = b.try_apply_all(op::cnot(0, 1));
        CHECK(e && e->kind == OperationError::InvalidArity && e->a == 2);
    }
    {  // invalid_target_returns_error (src/register.rs:437-445)
        Register r = Register::new_({false, false});
        auto e = r.try_apply(op::cnot(1, 2));
        CHECK(e && (*e == OperationError{OperationError::InvalidTarget, 2, 0}));
        CHECK(r.try_apply(op::cnot(1, 1)).has_value());
        CHECK(!r.try_apply(op::cnot(0, 1)).has_value());
    }
    {  // teleportation through QuantumCircuit / apply_circuit
        for (int k = 0; k < 10; k++) {
            const double th = 0.3 * k, ph = 0.7 * k;
            const c64 a(std::cos(th / 2), 0), b = std::polar(std::sin(th / 2), ph);
            Register r = Register::new_({false, false, false});
            r.seed(k);
            std::vector<c64> st(8, 0.0);
            st[0] = a;
            st[1] = b;
            r.set_state(st);
            QuantumCircuit c;
            c.add_operation(op::hadamard(2));
            c.add_operation(op::cnot(2, 1));
            c.add_operation(op::cnot(0, 1));
            c.add_operation(op::hadamard(0));
            c.add_measurement(1);
            c.add_measurement(0);
            c.add_conditional_operation(op::not_(2), {{1, true}});
            c.add_conditional_operation(op::pauli_z(2), {{0, true}});
            r.apply_circuit(c, k % 2);
            const auto s = r.state();
            c64 al = 0, be = 0;
            for (size_t i = 0; i < 8; i++) ((i >> 2) & 1 ? be : al) += s[i];
            const double nrm = std::sqrt(std::norm(al) + std::norm(be));
            CHECK(std::abs(al / nrm - a) < 1e-8 && std::abs(be / nrm - b) < 1e-8);
        }
    }
    {  // an OpenQASM file: a Bell pair from a user-defined Hadamard
        const std::string path = tmp + "/facade_bell.qasm";
        std::ofstream(path) << "OPENQASM 2.0;\ngate hh a { U(pi/2, 0, pi) a; }\nqreg q[2];\nhh q[0];\nCX q[0], q[1];\n";
        auto r = openqasm::run_openqasm(path);
        CHECK(r.first.has_value());
        if (r.first) {
            const auto p = r.first->qregs.at("q").probabilities();
            // angles pass through f32 as in the reference (src/openqasm.rs:98)
            CHECK(std::abs(p[0] - 0.5) < 1e-7 && std::abs(p[3] - 0.5) < 1e-7);
        }
        std::ofstream(path) << "OPENQASM 2.0;\nqreg q[2];\nnope q[0];\n";
        auto bad = openqasm::run_openqasm(path);
        CHECK(!bad.first && bad.second && bad.second->kind == openqasm::OpenQASMError::OpenQASMParseError);
    }
    std::printf(failures ? "facade tests: %d FAILED\n" : "facade tests: all passed%.0d\n", failures);
    return failures ? 1 : 0;
}
