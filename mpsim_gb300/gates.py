"""Gate library with mpsim's constructors and conventions (mpsim/gates.py).

Gates are host-side NumPy tensors wrapped in a small ``Node`` (the reference
returns ``tensornetwork.Node`` objects; this package does not depend on
TensorNetwork, and every entry point also accepts a bare array, a torch tensor
or any object with a ``.tensor`` attribute, so real TensorNetwork nodes work
too).  Matrices, dtypes and names follow the reference exactly, including its
quirks: ``cnot``/``swap`` are float64 (gates.py:195-221), ``haar_random_unitary``
is complex128 (gates.py:248-286) and ``rgate`` multiplies ``my*Y*mz*Z``
(gates.py:162).  The device path casts every gate to complex64.
"""

from __future__ import annotations

from copy import deepcopy
from typing import Optional

import numpy as np


class Node:
    """A gate tensor with one dangling edge per axis (TensorNetwork-like)."""

    def __init__(self, tensor, name: Optional[str] = None):
        self.tensor = np.asarray(tensor)
        self.name = name if name is not None else "__unnamed_node__"

    @property
    def shape(self):
        return self.tensor.shape

    @property
    def edges(self):
        return list(range(self.tensor.ndim))

    def get_all_edges(self):
        return self.edges

    def get_all_dangling(self):
        return self.edges

    def get_all_nondangling(self):
        return []

    def has_nondangling_edge(self):
        return False

    def __str__(self):
        return self.name

    def __repr__(self):
        return f"Node({self.name}, shape={self.shape})"


def gate_tensor(gate) -> np.ndarray:
    """The ndarray behind a gate given as Node / tn.Node / ndarray / tensor."""
    if hasattr(gate, "tensor"):
        t = gate.tensor
    else:
        t = gate
    if hasattr(t, "detach"):
        t = t.detach().cpu().numpy()
    return np.asarray(t)


def _square(gate) -> np.ndarray:
    g = gate_tensor(gate)
    if g.ndim > 2:
        if len(set(g.shape)) != 1:
            raise ValueError("Gate shape should be of the form (d, d, ..., d).")
        dim = int(np.sqrt(g.size))
        g = np.reshape(g, (dim, dim))
    return g


def is_unitary(gate) -> bool:
    """gates.py:15-33 (allclose with atol=1e-5)."""
    if not (isinstance(gate, (np.ndarray, Node)) or hasattr(gate, "tensor")):
        raise TypeError("Invalid type for gate.")
    g = _square(gate)
    # np.allclose(g^H g, I, atol=1e-5) (rtol 1e-5), written out: the same test
    # without allclose's per-call overhead (it runs once per applied gate)
    eye = np.identity(g.shape[0])
    return bool(np.all(np.abs(g.conj().T @ g - eye) <= 1e-5 + 1e-5 * eye))


def is_hermitian(gate) -> bool:
    """gates.py:36-52."""
    if not (isinstance(gate, (np.ndarray, Node)) or hasattr(gate, "tensor")):
        raise TypeError("Invalid type for gate.")
    g = _square(gate)
    return bool(np.allclose(g.conj().T, g, atol=1e-5))


def is_projector(gate) -> bool:
    """gates.py:55-70."""
    if not (isinstance(gate, (np.ndarray, Node)) or hasattr(gate, "tensor")):
        raise TypeError("Invalid type for gate.")
    return bool(np.linalg.matrix_rank(_square(gate)) == 1)


zero_state = np.array([1.0, 0.0], dtype=np.complex64)
one_state = np.array([0.0, 1.0], dtype=np.complex64)
# NumPy 1 kept these complex64 (value-based casting); NumPy 2 would promote.
plus_state = (1.0 / np.sqrt(2) * (zero_state + one_state)).astype(np.complex64)


def computational_basis_state(state: int, dim: int = 2) -> Node:
    """gates.py:79-101."""
    if state < 0:
        raise ValueError(f"Argument state should be positive but is {state}.")
    if dim < 0:
        raise ValueError(f"Argument dim should be positive but is {dim}.")
    if state >= dim:
        raise ValueError(f"Requires state < dim but state = {state} and dim = {dim}.")
    v = np.zeros((dim,))
    v[state] = 1.0
    return Node(v, name=f"|{state}>")


_hmatrix = (1 / np.sqrt(2) * np.array([[1.0, 1.0], [1.0, -1.0]])).astype(np.complex64)
_imatrix = np.array([[1.0, 0.0], [0.0, 1.0]], dtype=np.complex64)
_xmatrix = np.array([[0.0, 1.0], [1.0, 0.0]], dtype=np.complex64)
_ymatrix = np.array([[0.0, -1j], [1j, 0.0]], dtype=np.complex64)
_zmatrix = np.array([[1.0, 0.0], [0.0, -1.0]], dtype=np.complex64)


def igate() -> Node:
    return Node(deepcopy(_imatrix), name="igate")


def xgate() -> Node:
    return Node(deepcopy(_xmatrix), name="xgate")


def ygate() -> Node:
    return Node(deepcopy(_ymatrix), name="ygate")


def zgate() -> Node:
    return Node(deepcopy(_zmatrix), name="zmat")


def hgate() -> Node:
    return Node(deepcopy(_hmatrix), name="hgate")


def rgate(seed: Optional[int] = None, angle_scale: float = 1.0) -> Node:
    """gates.py:141-164, including its ``if seed:`` and ``my*Y*mz*Z`` term."""
    from scipy.linalg import expm
    if seed:
        np.random.seed(seed)
    theta, alpha, phi = np.random.rand(3) * 2 * np.pi
    mx = np.sin(alpha) * np.cos(phi)
    my = np.sin(alpha) * np.sin(phi)
    mz = np.cos(alpha)
    theta *= angle_scale
    unitary = expm(-1j * theta * (mx * _xmatrix + my * _ymatrix * mz * _zmatrix))
    return Node(unitary)


def computational_basis_projector(state: int, dim: int = 2) -> Node:
    """gates.py:168-191."""
    if state < 0:
        raise ValueError(f"Argument state should be positive but is {state}.")
    if dim < 0:
        raise ValueError(f"Argument dim should be positive but is {dim}.")
    if state >= dim:
        raise ValueError(f"Requires state < dim but state = {state} and dim = {dim}.")
    p = np.zeros((dim, dim))
    p[state, state] = 1.0
    return Node(p, name=f"|{state}><{state}|")


_cnot_matrix = np.reshape(np.array([[1.0, 0.0, 0.0, 0.0],
                                    [0.0, 1.0, 0.0, 0.0],
                                    [0.0, 0.0, 0.0, 1.0],
                                    [0.0, 0.0, 1.0, 0.0]]), (2, 2, 2, 2))
_swap_matrix = np.reshape(np.array([[1.0, 0.0, 0.0, 0.0],
                                    [0.0, 0.0, 1.0, 0.0],
                                    [0.0, 1.0, 0.0, 0.0],
                                    [0.0, 0.0, 0.0, 1.0]]), (2, 2, 2, 2))


def cnot() -> Node:
    return Node(deepcopy(_cnot_matrix), name="cnot")


def swap() -> Node:
    return Node(deepcopy(_swap_matrix), name="swap")


def cphase(exp: float) -> Node:
    """gates.py:224-232."""
    m = np.array([[1.0, 0.0, 0.0, 0.0],
                  [0.0, 1.0, 0.0, 0.0],
                  [0.0, 0.0, 1.0, 0.0],
                  [0.0, 0.0, 0.0, np.exp(1j * 2 * np.pi * exp)]], dtype=np.complex64)
    return Node(np.reshape(m, (2, 2, 2, 2)), name="cphase")


def random_two_qubit_gate(seed: Optional[int] = None) -> Node:
    """gates.py:235-245."""
    from scipy.stats import unitary_group
    if seed:
        np.random.seed(seed)
    u = unitary_group.rvs(dim=4)
    return Node(deepcopy(np.reshape(u, (2, 2, 2, 2))), name="R2Q")


def haar_random_matrix(nqudits: int = 2, qudit_dimension: int = 2,
                       seed: Optional[int] = None) -> np.ndarray:
    """Haar-random unitary as a (D, D) complex128 matrix, D = d**nqudits.

    The algorithm of gates.py:248-286 (Mezzadri, arXiv:math-ph/0609050): a
    ``RandomState(seed)`` complex Gaussian matrix (real and imaginary parts
    from one ``randn(D, D, 2)`` draw, scaled by 1/sqrt(2)), its QR
    factorisation, and Q times the phases of diag(R).
    """
    rng = np.random.RandomState(seed)
    dim = qudit_dimension ** nqudits
    z = rng.randn(dim, dim, 2)
    mat = (z[..., 0] + 1j * z[..., 1]) / np.sqrt(2)
    q, r = np.linalg.qr(mat)
    ph = np.diag(r).copy()
    ph /= np.abs(ph)
    return q * ph


def haar_random_unitary(nqudits: int = 2, qudit_dimension: int = 2,
                        name: str = "Haar", seed: Optional[int] = None) -> Node:
    """gates.py:248-286, returned as a (d,)*2n tensor node."""
    m = haar_random_matrix(nqudits, qudit_dimension, seed)
    return Node(np.reshape(m, [qudit_dimension] * 2 * nqudits), name=name)
