"""Stand-ins for the few Cirq objects the reference's simulator and circuit
tests use (Cirq is not installed): a line qubit, an operation exposing the
attributes mps_operation_from_gate_operation reads (``qubits``,
``_has_unitary_``, ``_unitary_``; mpsim/mpsim_cirq/circuits.py:12-43), and the
unitaries of Cirq's standard gates in Cirq's basis order (first qubit most
significant)."""
import numpy as np

I2 = np.eye(2, dtype=np.complex128)
X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Y = np.array([[0, -1j], [1j, 0]])
Z = np.diag([1.0, -1.0]).astype(np.complex128)
H = np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2)
S = np.diag([1, 1j])
T = np.diag([1, np.exp(1j * np.pi / 4)])
CNOT = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)
CZ = np.diag([1, 1, 1, -1]).astype(np.complex128)
SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)
ISWAP = np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]])


def czpow(t):
    return np.diag([1, 1, 1, np.exp(1j * np.pi * t)])


def fsim(theta, phi):
    c, s = np.cos(theta), -1j * np.sin(theta)
    return np.array([[1, 0, 0, 0], [0, c, s, 0], [0, s, c, 0], [0, 0, 0, np.exp(-1j * phi)]])


class LineQubit:
    def __init__(self, x):
        self.x = x

    def __hash__(self):
        return hash(("q", self.x))

    def __eq__(self, other):
        return isinstance(other, LineQubit) and other.x == self.x

    def __lt__(self, other):
        return self.x < other.x


class Op:
    """The parts of a cirq.GateOperation that the conversion reads."""

    def __init__(self, matrix, *qubits):
        self.qubits = tuple(qubits)
        self._m = None if matrix is None else np.asarray(matrix)

    def _has_unitary_(self):
        return self._m is not None

    def _unitary_(self):
        return self._m.copy()


