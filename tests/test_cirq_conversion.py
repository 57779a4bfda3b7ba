"""mps_operation_from_gate_operation (mpsim/mpsim_cirq/circuits.py:12-43) on
duck-typed operations, restating circuits_test.py's conversion checks; no GPU
is needed."""
import numpy as np
import pytest

from cirq_like import CNOT, LineQubit, Op
from mpsim_gb300.core import CannotConvertToMPSOperation, MPSOperation
from mpsim_gb300.mpsim_cirq import mps_operation_from_gate_operation


def test_operation_without_unitary_cannot_convert():
    q = LineQubit(0)
    with pytest.raises(CannotConvertToMPSOperation):
        mps_operation_from_gate_operation(Op(None, q), {q: 0})


def test_conversion_of_nonlocal_cnot():
    """circuits_test.py: a CNOT on qubits (0, 2) becomes a (2,2,2,2) node on
    indices (0, 2); the reversed order keeps the operation's qubit order."""
    q = [LineQubit(i) for i in range(3)]
    index = {qb: i for i, qb in enumerate(q)}
    op = mps_operation_from_gate_operation(Op(CNOT, q[2], q[0]), index)
    assert isinstance(op, MPSOperation)
    assert op.qudit_indices == (2, 0) and op.qudit_dimension == 2
    assert op.tensor(reshape_to_square_matrix=False).shape == (2, 2, 2, 2)
    assert np.allclose(op.tensor(), CNOT)
    assert MPSOperation.from_gate_operation is not None
