// quaru.hpp — C++17 host API mirroring Quaru's Rust API over the C ABI (quaru_gpu.h).
//
// Register (src/register.rs), Operation and the gate constructors
// (src/operation.rs), QuantumCircuit (src/operation.rs:79-322) and
// openqasm::{run_openqasm, u} (src/openqasm.rs). try_* methods return an
// std::optional<OperationError> (empty = Ok), the plain methods throw
// std::runtime_error where Rust panics. Measurement draws come from a
// per-register std::mt19937_64 (seedable) because the reference's thread_rng
// cannot be seeded. Header-only; link with -lquaru_gb300.
#pragma once

#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <optional>
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../quaru_gpu.h"

namespace quaru {

using c64 = std::complex<double>;

// ------------------------------------------------------------------ errors
struct OperationError {  // src/register.rs:10-20
    enum Kind { InvalidTarget, InvalidDimensions, InvalidArity, InvalidQubit } kind;
    size_t a = 0, b = 0;
    bool operator==(const OperationError& o) const { return kind == o.kind && a == o.a && b == o.b; }
};

namespace detail {
inline std::optional<OperationError> status(int rc, const size_t* err) {
    switch (rc) {
        case QS_OK: return std::nullopt;
        case QS_INVALID_TARGET: return OperationError{OperationError::InvalidTarget, err[0], 0};
        case QS_INVALID_DIMENSIONS: return OperationError{OperationError::InvalidDimensions, err[0], err[1]};
        case QS_INVALID_ARITY: return OperationError{OperationError::InvalidArity, err[0], 0};
        case QS_INVALID_QUBIT: return OperationError{OperationError::InvalidQubit, err[0], 0};
        default: throw std::runtime_error(std::string("quaru_gb300: ") + qs_last_error());
    }
}
inline void check(int rc) {
    if (rc != QS_OK) throw std::runtime_error(std::string("quaru_gb300: ") + qs_last_error());
}
}  // namespace detail

// ------------------------------------------------------------------ Operation
class Operation {  // src/operation.rs:49-70
   public:
    Operation(std::vector<c64> matrix, std::vector<size_t> targets)
        : m_(std::move(matrix)), t_(std::move(targets)) {}
    // Operation::new: nullopt unless the matrix is 2^k x 2^k (given as dim x dim row-major).
    static std::optional<Operation> create(std::vector<c64> matrix, size_t dim, std::vector<size_t> targets) {
        if (targets.size() >= 63 || dim != (size_t(1) << targets.size()) || matrix.size() != dim * dim)
            return std::nullopt;
        return Operation(std::move(matrix), std::move(targets));
    }
    const std::vector<c64>& matrix() const { return m_; }
    const std::vector<size_t>& targets() const { return t_; }
    size_t arity() const { return t_.size(); }
    size_t dim() const { return size_t(1) << t_.size(); }
    bool operator==(const Operation& o) const { return m_ == o.m_ && t_ == o.t_; }

   private:
    std::vector<c64> m_;
    std::vector<size_t> t_;
};

namespace operation {  // src/operation.rs:340-536
inline std::vector<c64> real(std::initializer_list<double> v) { return std::vector<c64>(v.begin(), v.end()); }
inline Operation identity(size_t t) { return Operation(real({1, 0, 0, 1}), {t}); }
inline Operation hadamard(size_t t) {
    const double h = 0.7071067811865476;
    return Operation(real({h, h, h, -h}), {t});
}
inline Operation hadamard_transform(const std::vector<size_t>& targets) {
    std::vector<c64> m = hadamard(targets[0]).matrix();
    size_t d = 2;
    for (size_t i = 1; i < targets.size(); i++) {  // kron(H, m)
        const auto h = hadamard(0).matrix();
        std::vector<c64> r(4 * d * d);
        for (size_t a = 0; a < 2; a++)
            for (size_t b = 0; b < 2; b++)
                for (size_t x = 0; x < d; x++)
                    for (size_t y = 0; y < d; y++) r[(a * d + x) * 2 * d + (b * d + y)] = h[a * 2 + b] * m[x * d + y];
        m.swap(r);
        d *= 2;
    }
    return Operation(m, targets);
}
inline Operation cnot(size_t control, size_t target) {
    return Operation(real({1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0}), {target, control});
}
inline Operation to_quantum_gate(const std::function<size_t(size_t)>& f, std::vector<size_t> targets) {
    const size_t n = size_t(1) << targets.size();
    std::vector<c64> m(n * n, 0.0);
    for (size_t c = 0; c < n; c++) m[f(c) * n + c] = 1.0;
    return Operation(m, std::move(targets));
}
inline Operation to_controlled(const Operation& op, size_t control) {
    const size_t d = op.dim(), n = 2 * d;
    std::vector<c64> m(n * n, 0.0);
    for (size_t i = 0; i < d; i++) m[i * n + i] = 1.0;
    for (size_t i = 0; i < d; i++)
        for (size_t j = 0; j < d; j++) m[(i + d) * n + j + d] = op.matrix()[i * d + j];
    auto t = op.targets();
    t.push_back(control);
    return Operation(m, t);
}
inline Operation swap(size_t a, size_t b) {
    return Operation(real({1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, 1}), {a, b});
}
inline Operation phase(size_t t) { return Operation({1.0, 0.0, 0.0, c64(0, 1)}, {t}); }
inline Operation not_(size_t t) { return Operation(real({0, 1, 1, 0}), {t}); }
inline Operation pauli_y(size_t t) { return Operation({0.0, c64(0, -1), c64(0, 1), 0.0}, {t}); }
inline Operation pauli_z(size_t t) { return Operation(real({1, 0, 0, -1}), {t}); }
inline Operation cnx(const std::vector<size_t>& controls, size_t target) {
    std::vector<size_t> t{target};
    t.insert(t.end(), controls.begin(), controls.end());
    const size_t n = size_t(1) << t.size();
    std::vector<c64> m(n * n, 0.0);
    for (size_t i = 0; i + 2 < n; i++) m[i * n + i] = 1.0;
    m[(n - 1) * n + n - 2] = 1.0;
    m[(n - 2) * n + n - 1] = 1.0;
    return Operation(m, t);
}
inline Operation cnz(const std::vector<size_t>& controls, size_t target) {
    std::vector<size_t> t{target};
    t.insert(t.end(), controls.begin(), controls.end());
    const size_t n = size_t(1) << t.size();
    std::vector<c64> m(n * n, 0.0);
    for (size_t i = 0; i + 1 < n; i++) m[i * n + i] = 1.0;
    m[(n - 1) * n + n - 1] = -1.0;
    return Operation(m, t);
}
}  // namespace operation

namespace openqasm {
// openqasm::u (src/openqasm.rs:145-163)
inline std::optional<Operation> u(double theta, double phi, double lambda, size_t target) {
    const double c = std::cos(theta / 2), s = std::sin(theta / 2);
    auto e = [](double x) { return c64(std::cos(x), std::sin(x)); };
    return Operation::create({e(-(phi + lambda) / 2) * c, -e(-(phi - lambda) / 2) * s, e((phi - lambda) / 2) * s,
                              e((phi + lambda) / 2) * c},
                             2, {target});
}
}  // namespace openqasm

// ------------------------------------------------------------------ QuantumCircuit
class QuantumCircuit {  // src/operation.rs:79-322 (builder and accessors)
   public:
    void add_operation(Operation op) {
        for (size_t t : op.targets())
            for (size_t m : meas_)
                if (t == m) throw std::runtime_error("Cannot add operation after measurement");
        if (!cond_.empty()) throw std::runtime_error("Cannot add operation after conditional operation (yet...)");
        ops_.push_back(std::move(op));
    }
    void add_measurement(size_t target) {
        for (size_t m : meas_)
            if (m == target) throw std::runtime_error("Cannot add measurement after measurement");
        meas_.push_back(target);
    }
    void add_conditional_operation(Operation op, std::vector<std::pair<size_t, bool>> condition) {
        for (size_t t : op.targets())
            for (size_t m : meas_)
                if (t == m) throw std::runtime_error("Cannot add operation after measurement");
        for (auto& c : condition) {
            bool found = false;
            for (size_t m : meas_) found |= (m == c.first);
            if (!found) throw std::runtime_error("Condition must be a measurement");
        }
        cond_.push_back({std::move(op), std::move(condition)});
    }
    const std::vector<Operation>& get_operations() const { return ops_; }
    const std::vector<size_t>& get_measurement_targets() const { return meas_; }
    const std::vector<std::pair<Operation, std::vector<std::pair<size_t, bool>>>>& get_conditional_operations() const {
        return cond_;
    }
    void clear_operations() { ops_.clear(); }

   private:
    std::vector<Operation> ops_;
    std::vector<size_t> meas_;
    std::vector<std::pair<Operation, std::vector<std::pair<size_t, bool>>>> cond_;
};

// ------------------------------------------------------------------ Register
class Register {  // src/register.rs:22-413
   public:
    static Register new_(const std::vector<bool>& bits, int precision = QS_PREC_C128) {
        std::vector<uint8_t> b(bits.begin(), bits.end());
        qs_register* h = nullptr;
        detail::check(qs_register_new(b.data(), b.size(), precision, &h));
        return Register(h);
    }
    static Register from_int(size_t n, size_t k, int precision = QS_PREC_C128) {
        qs_register* h = nullptr;
        detail::check(qs_register_from_int(n, k, precision, &h));
        return Register(h);
    }
    // Register::try_from_qubits: each qubit is a pair of amplitudes.
    static std::pair<std::optional<Register>, std::optional<OperationError>> try_from_qubits(
        const std::vector<std::pair<c64, c64>>& qubits, int precision = QS_PREC_C128) {
        std::vector<double> q;
        for (auto& p : qubits) q.insert(q.end(), {p.first.real(), p.first.imag(), p.second.real(), p.second.imag()});
        qs_register* h = nullptr;
        size_t err[3] = {0, 0, 0};
        auto e = detail::status(qs_register_try_from_qubits(q.data(), qubits.size(), precision, &h, err), err);
        if (e) return {std::nullopt, e};
        return {Register(h), std::nullopt};
    }
    static Register from_qubits(const std::vector<std::pair<c64, c64>>& qubits) {
        auto r = try_from_qubits(qubits);
        if (!r.first) throw std::runtime_error("Incorrect input qubits");
        return std::move(*r.first);
    }

    Register clone() const {
        qs_register* h = nullptr;
        detail::check(qs_register_clone(h_.get(), &h));
        return Register(h);
    }
    size_t size() const { return qs_register_size(h_.get()); }
    void seed(uint64_t s) { rng_.seed(s); }
    void set_arith(int arith) { detail::check(qs_register_set_arith(h_.get(), arith)); }
    qs_register* handle() const { return h_.get(); }

    std::optional<OperationError> try_apply_fast(const Operation& op) {
        size_t err[3] = {0, 0, 0};
        return detail::status(qs_try_apply_fast(h_.get(), reinterpret_cast<const double*>(op.matrix().data()),
                                                op.dim(), op.dim(), op.targets().data(), op.arity(), err),
                              err);
    }
    std::optional<OperationError> try_apply(const Operation& op) { return try_apply_fast(op); }
    Register& apply(const Operation& op) {
        if (try_apply_fast(op)) throw std::runtime_error("Could not apply operation");
        return *this;
    }
    std::optional<OperationError> try_apply_all(const Operation& op) {
        size_t err[3] = {0, 0, 0};
        return detail::status(qs_try_apply_all(h_.get(), reinterpret_cast<const double*>(op.matrix().data()),
                                               op.dim(), op.dim(), op.arity(), err),
                              err);
    }
    Register& apply_all(const Operation& op) {
        if (try_apply_all(op)) throw std::runtime_error("Could not apply operation");
        return *this;
    }
    // Several gates in one call (fuse: 0 one sweep per gate, 1 cache-blocked stages, 2 dense blocks).
    std::optional<OperationError> try_apply_gates(const std::vector<Operation>& ops, int fuse = 0) {
        std::vector<qs_gate> g;
        for (auto& op : ops)
            g.push_back({op.arity(), op.targets().data(), reinterpret_cast<const double*>(op.matrix().data())});
        qs_circuit_options o{fuse, 5, 0, 0};
        size_t err[3] = {0, 0, 0};
        return detail::status(qs_apply_circuit(h_.get(), g.data(), g.size(), &o, err), err);
    }

    std::pair<bool, std::optional<OperationError>> try_measure(size_t target) {
        int out = 0;
        size_t err[3] = {0, 0, 0};
        const double x = std::uniform_real_distribution<double>(0.0, 1.0)(rng_);
        auto e = detail::status(qs_try_measure(h_.get(), target, x, &out, nullptr, nullptr, err), err);
        return {out != 0, e};
    }
    bool measure(size_t target) {
        auto r = try_measure(target);
        if (r.second) throw std::runtime_error("Could not measure bit");
        return r.first;
    }

    // Register::apply_circuit (src/register.rs:345-369) and measure_circuit (:371-377).
    std::vector<std::pair<size_t, bool>> apply_circuit(const QuantumCircuit& c, int fuse = 0) {
        if (!c.get_operations().empty() && try_apply_gates(c.get_operations(), fuse))
            throw std::runtime_error("Could not apply operation");
        std::vector<std::pair<size_t, bool>> m;
        if (!c.get_measurement_targets().empty()) m = measure_circuit(c);
        for (auto& co : c.get_conditional_operations()) {
            bool ok = true;
            for (auto& cond : co.second) {
                bool hit = false;
                for (auto& x : m) hit |= (x == cond);
                ok &= hit;
            }
            if (ok) apply(co.first);
        }
        return m;
    }
    std::vector<std::pair<size_t, bool>> measure_circuit(const QuantumCircuit& c) {
        std::vector<std::pair<size_t, bool>> m;
        for (size_t t : c.get_measurement_targets()) m.push_back({t, measure(t)});
        return m;
    }

    std::vector<c64> state() const {  // `pub state`
        std::vector<c64> s(size_t(1) << size());
        detail::check(qs_get_state(h_.get(), reinterpret_cast<double*>(s.data())));
        return s;
    }
    void set_state(const std::vector<c64>& s) {
        detail::check(qs_set_state(h_.get(), reinterpret_cast<const double*>(s.data())));
    }
    std::vector<double> probabilities() const {
        std::vector<double> p(size_t(1) << size());
        detail::check(qs_probabilities(h_.get(), p.data()));
        return p;
    }
    void print_probabilities() const {
        const auto p = probabilities();
        for (size_t i = 0; i < p.size(); i++) std::printf("%s: %.17g%%\n", bin(i).c_str(), p[i] * 100.0);
    }
    void print_nonzero_probabilities() const {
        const auto p = probabilities();
        for (size_t i = 0; i < p.size(); i++)
            if (p[i] > 0.0) std::printf("%s: %.17g%%\n", bin(i).c_str(), p[i] * 100.0);
    }
    bool operator==(const Register& o) const {  // PartialEq, tolerance 1e-8
        int eq = 0;
        detail::check(qs_register_eq(h_.get(), o.h_.get(), 1e-8, &eq));
        return eq != 0;
    }

    explicit Register(qs_register* h) : h_(h, &qs_register_free), rng_(std::random_device{}()) {}

   private:
    std::string bin(size_t i) const {
        std::string s(size(), '0');
        for (size_t b = 0; b < s.size(); b++)
            if (i >> b & 1) s[s.size() - 1 - b] = '1';
        return s;
    }
    std::unique_ptr<qs_register, void (*)(qs_register*)> h_;
    std::mt19937_64 rng_;
};

// ------------------------------------------------------------------ openqasm
namespace openqasm {
struct OpenQASMError {
    enum Kind { OpenQASMParseError, OpenQASMRunError } kind;
    std::string message;
};
struct OpenQASMResult {
    std::map<std::string, Register> qregs;
    std::map<std::string, std::vector<bool>> cregs;
};
// openqasm::run_openqasm (src/openqasm.rs:52-142); `seed` drives measurement draws.
inline std::pair<std::optional<OpenQASMResult>, std::optional<OpenQASMError>> run_openqasm(const std::string& path,
                                                                                           uint64_t seed = 0) {
    qs_qasm_result* r = nullptr;
    const int rc = qs_qasm_run_file(path.c_str(), seed, QS_PREC_C128, &r);
    if (rc == QS_QASM_PARSE_ERROR || rc == QS_QASM_RUN_ERROR)
        return {std::nullopt, OpenQASMError{rc == QS_QASM_PARSE_ERROR ? OpenQASMError::OpenQASMParseError
                                                                      : OpenQASMError::OpenQASMRunError,
                                            qs_last_error()}};
    detail::check(rc);
    OpenQASMResult out;
    for (size_t i = 0; i < qs_qasm_qreg_count(r); i++) {
        qs_register* h = nullptr;
        detail::check(qs_register_clone(qs_qasm_qreg(r, i), &h));
        out.qregs.emplace(qs_qasm_qreg_name(r, i), Register(h));
    }
    for (size_t i = 0; i < qs_qasm_creg_count(r); i++) {
        std::vector<uint8_t> b(qs_qasm_creg_size(r, i));
        qs_qasm_creg_bits(r, i, b.data());
        out.cregs.emplace(qs_qasm_creg_name(r, i), std::vector<bool>(b.begin(), b.end()));
    }
    qs_qasm_free(r);
    return {std::move(out), std::nullopt};
}
}  // namespace openqasm

}  // namespace quaru
