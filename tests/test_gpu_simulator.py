"""MPSimulator and the Cirq operation conversion, restating the reference's
mpsim/mpsim_cirq/simulator_test.py (:16-19, 22-144, 262-331) and
circuits_test.py without Cirq (not installed): operations are duck-typed
objects with ``qubits``, ``_has_unitary_`` and ``_unitary_`` -- the three
attributes mps_operation_from_gate_operation (mpsim/mpsim_cirq/circuits.py:
12-43) reads -- and Cirq's dense simulator is replaced by the dense oracle
(oracle/dense.py).  Comparisons are np.allclose with atol=2e-6 instead of
the reference tests' default 1e-8: the reference silently promotes its state
to complex128 on contact with Cirq's complex128 unitaries, while this build
stores complex64 throughout, whose rounding leaves ~1e-8 where the exact
amplitude is 0 after 25 moments of gates.
"""
import numpy as np
import pytest

from cirq_like import (CNOT, CZ, H, I2, ISWAP, SWAP, S, T, X, Y, Z, LineQubit, Op, czpow,
                       fsim)
from mpsim_gb300.core import MPS
from mpsim_gb300.mpsim_cirq import MPSimulator, mps_operation_from_gate_operation
from oracle.dense import DenseState

pytestmark = pytest.mark.gpu


def convert(ops):
    qubits = sorted({q for op in ops for q in op.qubits})
    index = {q: i for i, q in enumerate(qubits)}
    return [mps_operation_from_gate_operation(op, index) for op in ops], len(qubits)


def dense_of(ops, n):
    st = DenseState(n)
    qubits = sorted({q for op in ops for q in op.qubits})
    index = {q: i for i, q in enumerate(qubits)}
    for op in ops:
        idx = [index[q] for q in op.qubits]
        if len(idx) == 1:
            st.apply_one(op._unitary_(), idx[0])
        else:
            st.apply_two(op._unitary_(), idx[0], idx[1])
    return st.vector()


def close(a, b):
    return np.allclose(a, b, atol=2e-6)


def simulate(ops, options=None):
    mops, n = convert(ops)
    mps = MPSimulator(options=options or {}).simulate(mops)
    assert isinstance(mps, MPS) and mps.nqudits == n
    return mps


def test_empty_program_raises(cuda):
    with pytest.raises(ValueError):
        MPSimulator().simulate([])


def test_identity_circuit(cuda):
    q = [LineQubit(i) for i in range(3)]
    ops = [Op(I2, qb) for qb in q]
    assert close(simulate(ops).wavefunction(), dense_of(ops, 3))


def test_bell_state(cuda):
    q = [LineQubit(0), LineQubit(1)]
    ops = [Op(H, q[0]), Op(CNOT, q[0], q[1])]
    assert close(simulate(ops).wavefunction(), np.array([1, 0, 0, 1]) / np.sqrt(2))


def test_bell_state_with_truncation(cuda):
    q = [LineQubit(0), LineQubit(1)]
    ops = [Op(H, q[0]), Op(CNOT, q[0], q[1])]
    res = simulate(ops, {"maxsvals": 1})
    assert close(res.wavefunction(), np.array([1, 0, 0, 0]) / np.sqrt(2))


@pytest.mark.parametrize("n", range(3, 10))
def test_ghz_circuits(cuda, n):
    q = [LineQubit(i) for i in range(n)]
    ops = [Op(H, q[0])] + [Op(CNOT, q[0], q[i]) for i in range(1, n)]   # non-local CNOTs
    assert close(simulate(ops).wavefunction(), dense_of(ops, n))


@pytest.mark.parametrize("n", range(3, 10))
def test_qft_circuits(cuda, n):
    q = [LineQubit(i) for i in range(n)]
    ops = []
    for i in range(n - 1, -1, -1):
        ops.append(Op(H, q[i]))
        for j in range(i - 1, -1, -1):
            ops.append(Op(czpow(2.0 ** (j - i)), q[j], q[i]))
    assert len(ops) == n * (n + 1) // 2
    assert close(simulate(ops).wavefunction(), dense_of(ops, n))


def test_three_qubit_gate_raises(cuda):
    q = [LineQubit(i) for i in range(3)]
    mops, _ = convert([Op(np.eye(8), *q)])
    with pytest.raises(ValueError):
        MPSimulator().simulate(mops)


@pytest.mark.parametrize("nqubits", [2, 4, 8])
def test_random_circuits(cuda, nqubits):
    """50 random circuits of 25 moments (op density ~1) over the gate domain
    of simulator_test.py:274-305, including non-adjacent two-qubit gates."""
    one = [X, Y, Z, H, S, T]
    two = [CNOT, CZ, SWAP, czpow(1.0), ISWAP, fsim(0.2, 0.3)]
    rng = np.random.default_rng(1)
    q = [LineQubit(i) for i in range(nqubits)]
    for _ in range(50):
        ops = []
        for _ in range(25):
            free = list(rng.permutation(nqubits))
            while free:
                if len(free) >= 2 and rng.random() < 0.5:
                    a, b = free.pop(), free.pop()
                    ops.append(Op(two[rng.integers(len(two))], q[a], q[b]))
                else:
                    ops.append(Op(one[rng.integers(len(one))], q[free.pop()]))
        # the state's qubit set must be all nqubits (conversion sorts qubits)
        assert len({qb for op in ops for qb in op.qubits}) == nqubits
        mps = simulate(ops)
        assert close(mps.wavefunction(), dense_of(ops, nqubits))


def test_custom_gate(cuda):
    rng = np.random.default_rng(1)
    z = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    u, _ = np.linalg.qr(z)
    q = [LineQubit(0), LineQubit(1)]
    ops = [Op(u, q[0], q[1])]
    assert close(simulate(ops).wavefunction(), dense_of(ops, 2))


def test_options_forwarded_and_norm(cuda):
    """Options reach MPS.apply (fraction as well as maxsvals), and a
    truncation-free random 1 x 5 circuit keeps unit norm, as the reference's
    one-dimensional supremacy-circuit test checks (simulator_test.py:97-110)."""
    rng = np.random.default_rng(4)
    q = [LineQubit(i) for i in range(5)]
    ops = []
    for layer in range(10):
        ops += [Op([X, Y, T][rng.integers(3)], qb) for qb in q]
        ops += [Op(CZ, q[i], q[i + 1]) for i in range(layer % 2, 4, 2)]
    res = simulate(ops)
    assert np.isclose(res.norm(), 1.0)
    cut = simulate(ops, {"fraction": 0.5})
    assert max(cut.bond_dimensions()) <= max(res.bond_dimensions())
    with pytest.raises(ValueError):
        simulate(ops, {"fraction": 0.5, "maxsvals": 2})
