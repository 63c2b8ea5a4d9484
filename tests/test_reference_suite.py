"""Quaru's own test suite, restated once and run on two backends.

Sources: tests/register_operation_tests.rs, src/register.rs:437-445,
examples/shors.rs:380-503, examples/grovers.rs:274-312,
examples/quantum_teleportation.rs:150-164, examples/superdense_coding.rs:84-97.
proptest strategies over small ranges are enumerated exhaustively; the
reference's unseeded thread_rng draws are replaced by seeded draws.
The "oracle" backend pins the CPU oracle to these known answers; the "gpu"
backend runs the same checks on the GB300 engine.
"""
from __future__ import annotations

import itertools
import math

import numpy as np
import pytest

from quaru_gb300 import operation as O
from quaru_gb300.operation import Operation
from tests.backends import Backend, equal_qubits

BACKENDS = ["oracle", pytest.param("gpu", marks=pytest.mark.gpu)]


@pytest.fixture(params=BACKENDS)
def B(request):
    return Backend(request.param)


def draws(seed: int, n: int) -> list[float]:
    return list(np.random.default_rng(seed).random(n))


# ---------------------------------------------------------------- tests/register_operation_tests.rs
def test_measure_on_zero_state_gives_false(B):  # :12-19
    for x in draws(1, 8) + [0.0, 0.999999999999]:
        assert B.new([False]).measure(0, x) is False


def test_from_qubits(B):  # :24-40
    s = 1.0 / math.sqrt(2.0)
    reg_q = B.try_from_qubits([[1, 0], [0, 1], [s, s]])
    reg = B.new([False, True, False]).apply(O.hadamard(2))
    assert equal_qubits(reg.state, reg_q.state)


def test_not_on_arbitrary_qubit(B):  # :44-50
    for i in range(3):
        for x in draws(i, 3):
            reg = B.new([False] * 3).apply(O.not_(i))
            assert reg.measure(i, x) is True


@pytest.mark.parametrize("n", [4, 8])
def test_measure_n_qubits_gives_same_result(B, n):  # :53-96 (all 2^n inputs)
    xs = draws(n, n)
    for bits in itertools.product([False, True], repeat=n):
        reg = B.new(list(bits))
        got = [reg.measure(q, xs[q]) for q in range(n)]
        assert got == list(bits)


def test_hadamard_hadamard_retains_original_state(B):  # :99-107
    for i in range(3):
        reg = B.new([False] * 3)
        expected = reg.state
        reg.apply(O.hadamard(i)).apply(O.hadamard(i))
        assert equal_qubits(reg.state, expected)


def test_any_entangled_bit_measure_same(B):  # :110-125
    xs = draws(7, 72)
    c = 0
    for i in range(6):
        for j in range(6):
            jj = (j + 1) % 6 if i == j else j
            reg = B.new([False] * 6)
            reg.apply(O.hadamard(i)).apply(O.cnot(i, jj))
            a = reg.measure(i, xs[c])
            b = reg.measure(jj, xs[c + 1])
            c += 2
            assert a == b


def test_first_bell_state_measure_equal(B):  # :129-140
    xs = draws(8, 10)
    for i in range(5):
        reg = B.new([False] * 6)
        reg.apply(O.hadamard(i)).apply(O.cnot(i, i + 1))
        assert reg.measure(i, xs[2 * i]) == reg.measure(i + 1, xs[2 * i + 1])


def test_arbitrary_unary_applied_twice_gives_equal(B):  # :143-152
    for i in range(6):
        for make in (O.hadamard, O.not_, O.identity):
            reg = B.new([False] * 6)
            expected = reg.state
            op = make(i)
            reg.apply(op).apply(op)
            assert equal_qubits(reg.state, expected)


def test_arbitrary_binary_applied_twice_gives_equal(B):  # :155-163
    for i in range(6):
        for j in range(6):
            if i == j:
                continue
            for make in (O.cnot, O.swap):
                reg = B.new([False] * 6)
                expected = reg.state
                op = make(i, j)
                reg.apply(op).apply(op)
                assert equal_qubits(reg.state, expected)


def test_swap_single_true_qubit(B):  # :166-181
    xs = draws(9, 5)
    for i in range(5):
        for j in range(5):
            if i == j:
                continue
            bits = [False] * 6
            bits[i] = True
            reg = B.new(bits).apply(O.swap(i, j))
            for k in range(5):
                assert reg.measure(k, xs[k]) == (k == j)


def test_toffoli(B):  # :184-208
    xs = draws(10, 6)
    for n in range(2, 7):
        for init in itertools.product([False, True], repeat=6):
            reg = B.new(list(init))
            reg.apply(O.cnx(list(range(n - 1)), n - 1))
            controls = all(reg.measure(i, xs[i]) for i in range(n - 1))
            target = reg.measure(n - 1, xs[n - 1])
            assert (target != init[n - 1]) if controls else (target == init[n - 1])


def test_apply_all(B):  # :211-219
    for n in range(2, 7):
        r1 = B.new([False] * n)
        r2 = B.new([False] * n)
        for i in range(n):
            r1.apply(O.hadamard(i))
        r2.apply_all(O.hadamard(0))
        assert equal_qubits(r1.state, r2.state)


def test_apply_all_panics_if_not_unary(B):  # :222-226
    for i, j in [(0, 1), (3, 5), (5, 0)]:
        for make in (O.cnot, O.swap):
            reg = B.new([False] * 6)
            with pytest.raises(Exception):
                reg.apply_all(make(i, j))
            with pytest.raises(Exception) as e:
                reg.try_apply_all(make(i, j))
            assert e.value.code == 3 and e.value.payload[0] == 2  # InvalidArity(2)


def test_invalid_target_returns_error(B):  # src/register.rs:437-445
    reg = B.new([False, False])
    with pytest.raises(Exception) as e:
        reg.try_apply(O.cnot(1, 2))
    assert e.value.code == 1 and e.value.payload == (2,)  # InvalidTarget(2)
    with pytest.raises(Exception) as e:
        reg.try_apply(O.cnot(1, 1))
    assert e.value.code == 1 and e.value.payload == (1,)
    reg.try_apply(O.cnot(0, 1))


def test_invalid_dimensions_and_qubits(B):
    reg = B.new([False] * 3)
    # a 2x2 matrix with two targets is the shape the reference's own check rejects (src/register.rs:141-145)
    with pytest.raises(Exception) as e:
        reg.try_apply(Operation(np.eye(2, dtype=complex), [0, 1]))
    assert e.value.code == 2 and e.value.payload == (2, 2)
    with pytest.raises(Exception) as e:
        B.try_from_qubits([[1, 0], [0.5, 0.5]])
    assert e.value.code == 4 and e.value.payload == (1,)


# ---------------------------------------------------------------- src/operation.rs tests (constructors)
def test_operations_shape_and_unitary():  # src/operation.rs:547-594
    ops = [O.identity(0), O.hadamard(0), O.cnot(0, 1), O.swap(0, 1), O.phase(0), O.not_(0), O.pauli_y(0),
           O.pauli_z(0)] + [O.cnx(list(range(c)), c) for c in range(1, 6)]
    for op in ops:
        m = op.matrix
        assert m.shape == (1 << op.arity(), 1 << op.arity())
        assert np.all(np.abs(m @ m.conj().T - np.eye(m.shape[0])) < 1e-8)
    assert np.all(np.abs(O.cnx([0], 1).matrix - O.cnot(0, 1).matrix) < 1e-8)


# ---------------------------------------------------------------- examples/shors.rs tests
def _modpow(base: int, exp: int, mod: int) -> int:  # src/math.rs:70-82
    result = 1
    while exp > 0:
        if exp % 2 == 1:
            result = (result * base) % mod
        exp //= 2
        base = base * base % mod
    return result


def u_gate(targets, modulus, a, i) -> Operation:  # examples/shors.rs:79-92
    a_pow = _modpow(a, 1 << i, modulus)
    return O.to_quantum_gate(lambda x: (x * a_pow) % modulus, targets)


def test_u_gate(B):  # examples/shors.rs:434-462 (exact permutation/0-1 gates)
    n = 4
    step = 1 if B.name == "oracle" else 3  # the GPU run covers every third modulus/base pair
    for modulus in range(1, 1 << n, 1):
        for base in range(0, 1 << n, step):
            for i in range(0, 1 << n, 5):
                gate = u_gate(list(range(n)), modulus, base, i)
                for inp in range(1 << n):
                    reg = B.from_int(n, inp).apply(gate)
                    ans = B.from_int(n, inp * _modpow(base, 1 << i, modulus) % modulus)
                    assert equal_qubits(reg.state, ans.state)


def qft(n: int) -> Operation:  # examples/shors.rs:363-373
    m = 1 << n
    idx = np.arange(m)
    mat = np.exp(2j * np.pi * ((np.outer(idx, idx) % m) / m)) / math.sqrt(m)
    return Operation.new(mat, list(range(n)))


def add_operation(a: int, targets) -> Operation:  # examples/shors.rs:466-483
    m = np.eye(1, dtype=complex)
    for i in range(len(targets)):
        em = np.array([[1, 0], [0, complex(math.cos(math.pi / 2 ** i * a), math.sin(math.pi / 2 ** i * a))]])
        m = np.kron(m, em)
    return Operation.new(m, list(targets))


def test_qft_add(B):  # examples/shors.rs:486-503
    n = 5
    g = qft(n)
    rng = range(0, 50) if B.name == "oracle" else range(0, 50, 7)
    for a in rng:
        add = add_operation(a, list(range(n)))
        for b in range(0, 50, 3):
            r1 = B.from_int(n, b % (1 << n)).apply(g).apply(add)
            r2 = B.from_int(n, (a + b) % (1 << n)).apply(g)
            assert equal_qubits(r1.state, r2.state)


def _limit_denominator(m: int, n: int, limit: int) -> tuple[int, int]:  # src/math.rs:55-66
    """The fraction closest to m/n with denominator at most `limit` (continued fractions)."""
    a, b, p, q, r, s = n, m % n, 1, 0, m // n, 1
    while 0 < b and q + a // b * s <= limit:
        a, b, p, q, r, s = b, a % b, r, s, p + a // b * r, q + a // b * s
    t, u = p + (limit - q) // s * r, q + (limit - q) // s * s
    return (r, s) if 2 * b * u <= n else (t, u)


def _qubits_for(number: int) -> int:  # ((number + 1) as f64).log2().ceil()
    return math.ceil(math.log2(number + 1))


def find_period_slow(B, number: int, a: int, draw) -> int:  # examples/shors.rs:232-291
    """3n qubits: H on the first 2n, |1> in the last n, a controlled U (x -> x a^2^i mod N) per
    counting qubit, the QFT on the counting qubits, measure them, continued fraction of res / 2^2n."""
    n = _qubits_for(number)
    reg = B.new([False] * (3 * n))
    reg.apply(O.hadamard_transform(list(range(2 * n))))
    reg.apply(O.not_(2 * n))
    targets = list(range(2 * n, 3 * n))
    for i in range(2 * n):
        reg.apply(O.to_controlled(u_gate(targets, number, a, i), i))
    reg.apply(qft(2 * n))
    res = 0
    for i in range(2 * n):
        if reg.measure(i, draw()):
            res |= 1 << i
    return _limit_denominator(res, 2 ** (2 * n) - 1, number - 1)[1]


def find_period_fast(B, number: int, a: int, draw) -> int:  # examples/shors.rs:293-357
    """n + 1 qubits: one control qubit reused 2n times (semiclassical QFT after Parker & Plenio,
    quant-ph/0001066): H, controlled U (x -> x a^2^(2n-1-i) mod N), the phase R(-2 pi sm), H,
    measure, reset to |0> on a 1."""
    n = _qubits_for(number)
    reg = B.new([False] * (n + 1))
    reg.apply(O.not_(1))
    res, sm = 0, 0.0
    targets = list(range(1, n + 1))
    for i in range(2 * n):
        reg.apply(O.hadamard(0))
        reg.apply(O.to_controlled(u_gate(targets, number, a, 2 * n - 1 - i), 0))
        phi = complex(math.cos(-2.0 * math.pi * sm), math.sin(-2.0 * math.pi * sm))
        reg.apply(Operation.new(np.array([[1.0, 0.0], [0.0, phi]], dtype=complex), [0]))
        reg.apply(O.hadamard(0))
        m = reg.measure(0, draw())
        sm /= 2.0
        if m:
            reg.apply(O.not_(0))
            res |= 1 << i
            sm += 0.25
    return _limit_denominator(res, 2 ** (2 * n) - 1, number - 1)[1]


def _draws(seed: int):
    rng = np.random.default_rng(seed)
    return lambda: float(rng.random())


@pytest.mark.parametrize("fast", [False, True])
def test_period_finder_working(B, fast):  # examples/shors.rs:380-410
    """For every N < 6 (slow) or < 15 (fast) and every a coprime to N: the period r of a^x mod N is
    a multiple of the found one in at least 15 of 20 runs (seeded draws)."""
    for number in range(2, 15 if fast else 6):
        for a in range(2, number):
            if math.gcd(number, a) != 1:
                continue
            period, a_pow = 1, a
            while a_pow != 1:
                a_pow = a_pow * a % number
                period += 1
            draw = _draws(1000 * number + a + (500 if fast else 0))
            ok = 0
            for _ in range(20):
                r = (find_period_fast if fast else find_period_slow)(B, number, a, draw)
                if period % r == 0:
                    ok += 1
            assert ok >= 15, (number, a, ok)


def shors(B, number: int, rng) -> int:  # examples/shors.rs:96-173 (fast period finder)
    if number % 2 == 0:
        return 2
    for k in range(2, int(math.log2(number)) + 1):  # prime powers c^k
        c = int(number ** (1.0 / k) + 1e-9)
        if c ** k == number:
            return c
    draw = _draws(int(rng.integers(1 << 30)))
    while True:
        a = int(rng.integers(2, number))
        k = math.gcd(a, number)
        if k != 1:
            return k
        r = find_period_fast(B, number, a, draw)
        if r % 2 == 0:
            k = _modpow(a, r // 2, number)
            if k != number - 1:
                for f in (math.gcd(k - 1, number), math.gcd(k + 1, number)):
                    if f != 1 and f != number:
                        return f


def test_shors_working(B):  # examples/shors.rs:412-420
    rng = np.random.default_rng(15)
    for number in (4, 6, 8, 9, 10, 12, 14, 15):
        r = shors(B, number, rng)
        assert number % r == 0 and 1 < r < number, (number, r)


# ---------------------------------------------------------------- examples/grovers.rs tests
def oracle_operation(regsize: int, winner: int, lst) -> Operation:  # examples/grovers.rs:181-203
    n = 1 << regsize
    d = np.ones(n)
    for i, item in enumerate(lst):
        if item == winner and i < n:
            d[i] = -1.0
    return Operation.new(np.diag(d).astype(complex), list(range(regsize)))


def diffusion_operation(regsize: int) -> Operation:  # examples/grovers.rs:208-218
    n = 1 << regsize
    d = -np.ones(n)
    d[0] = 1.0
    return Operation.new(np.diag(d).astype(complex), list(range(regsize)))


def _regsize(target):
    r = math.ceil(math.log2(target + 1))
    return max(r, 2)


def test_grover_oracle_operation(B):  # examples/grovers.rs:274-286
    for target in range(20):
        rs = _regsize(target)
        reg = B.new([False] * rs)
        reg.apply_all(O.hadamard(0))
        reg.apply(oracle_operation(rs, target, list(range(20))))
        assert np.signbit(reg.state[target].real)


def test_grover_diffuser_operation(B):  # examples/grovers.rs:292-311
    for target in range(20):
        rs = _regsize(target)
        reg = B.new([False] * rs)
        reg.apply_all(O.hadamard(0))
        reg.apply(oracle_operation(rs, target, list(range(20))))
        reg.apply_all(O.hadamard(0))
        reg.apply(diffusion_operation(rs))
        reg.apply_all(O.hadamard(0))
        st = reg.state
        for i in range(rs):
            if i != target:
                assert abs(st[i]) < abs(st[target])


# ---------------------------------------------------------------- examples/quantum_teleportation.rs
def get_state_of_qubit(state, n):  # examples/quantum_teleportation.rs:123-140
    alpha = beta = 0j
    for i, s in enumerate(state):
        if (i >> n) & 1:
            beta += s
        else:
            alpha += s
    p = abs(alpha) ** 2 + abs(beta) ** 2
    return np.array([alpha / math.sqrt(p), beta / math.sqrt(p)])


def test_quantum_teleportation(B):  # examples/quantum_teleportation.rs:150-156
    rng = np.random.default_rng(11)
    for _ in range(20):
        theta, phi = rng.uniform(0, math.pi), rng.uniform(0, 2 * math.pi)
        q0 = np.array([math.cos(theta / 2), math.sin(theta / 2) * complex(math.cos(phi), math.sin(phi))])
        reg = B.new([False] * 3)
        reg.state = np.kron(np.kron([1, 0], [1, 0]), q0)
        reg.apply(O.hadamard(2)).apply(O.cnot(2, 1)).apply(O.cnot(0, 1)).apply(O.hadamard(0))
        if reg.measure(1, rng.random()):
            reg.apply(O.not_(2))
        if reg.measure(0, rng.random()):
            reg.apply(O.pauli_z(2))
        assert equal_qubits(get_state_of_qubit(reg.state, 2), q0)


# ---------------------------------------------------------------- examples/superdense_coding.rs
def test_superdense_coding(B):  # examples/superdense_coding.rs:84-97
    xs = draws(12, 2)
    for a in (False, True):
        for b in (False, True):
            reg = B.new([False, False]).apply(O.hadamard(0)).apply(O.cnot(0, 1))
            if (a, b) == (False, False):
                reg.apply(O.identity(0))
            elif (a, b) == (False, True):
                reg.apply(O.not_(0))
            elif (a, b) == (True, False):
                reg.apply(O.pauli_z(0))
            else:
                reg.apply(O.pauli_z(0)).apply(O.not_(0))
            reg.apply(O.cnot(0, 1)).apply(O.hadamard(0))
            assert (reg.measure(0, xs[0]), reg.measure(1, xs[1])) == (a, b)
