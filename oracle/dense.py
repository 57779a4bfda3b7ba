"""Dense state-vector simulator (oracle; test infrastructure only).

The reference's own tests check MPS results against Cirq's dense simulator
(mpsim/mpsim_cirq/simulator_test.py:274-305, core_test.py:1225-1258).  Cirq is
not installed here, so this module restates the same dense evolution: a state
vector of d**n amplitudes, qudit 0 the most significant digit (the ordering
pinned by core_test.py:1187-1194).
"""

from __future__ import annotations

import numpy as np


class DenseState:
    def __init__(self, nqudits, qudit_dimension=2, dtype=np.complex128):
        self.n = nqudits
        self.d = qudit_dimension
        self.psi = np.zeros((qudit_dimension,) * nqudits, dtype=dtype)
        self.psi[(0,) * nqudits] = 1.0

    def apply_one(self, gate, i):
        u = np.asarray(gate, dtype=self.psi.dtype).reshape(self.d, self.d)
        self.psi = np.moveaxis(np.tensordot(u, self.psi, axes=([1], [i])), 0, i)

    def apply_two(self, gate, i, j):
        """gate[a', b', a, b]: a is qudit i, b is qudit j (any order)."""
        g = np.asarray(gate, dtype=self.psi.dtype).reshape((self.d,) * 4)
        out = np.tensordot(g, self.psi, axes=([2, 3], [i, j]))
        self.psi = np.moveaxis(out, [0, 1], [i, j])

    def vector(self):
        return self.psi.reshape(-1)
