"""Conversion of Cirq operations to MPS operations (mpsim/mpsim_cirq/circuits.py).

Cirq is optional: everything here imports without it, and the Cirq-specific
paths raise ImportError only when used without Cirq installed.
"""
from __future__ import annotations

from typing import Dict

import numpy as np

from mpsim_gb300.core import CannotConvertToMPSOperation, MPSOperation
from mpsim_gb300.gates import Node

try:  # pragma: no cover - cirq is not installed in the build image
    import cirq
except ImportError:
    cirq = None


def mps_operation_from_gate_operation(gate_operation, qudit_to_index_map: Dict) -> MPSOperation:
    """circuits.py:12-43: the operation's unitary reshaped to (2,)*2n."""
    num_qudits = len(gate_operation.qubits)
    qudit_dimension = 2
    qudit_indices = tuple(qudit_to_index_map[q] for q in gate_operation.qubits)
    if not gate_operation._has_unitary_():
        raise CannotConvertToMPSOperation(
            f"Cannot convert operation {gate_operation} into an MPS Operation"
            " because the operation does not have a unitary.")
    tensor = np.reshape(gate_operation._unitary_(), [qudit_dimension] * 2 * num_qudits)
    return MPSOperation(Node(tensor), qudit_indices, qudit_dimension)


MPSOperation.from_gate_operation = staticmethod(mps_operation_from_gate_operation)

if cirq is not None:  # pragma: no cover
    class MPSimCircuit(cirq.Circuit):
        """circuits.py:49-93."""

        def __init__(self, cirq_circuit, device=None, qubit_order=None):
            super().__init__(cirq_circuit)
            self._qudit_to_index_map = {q: i for i, q in enumerate(sorted(self.all_qubits()))}
            self._mps_operations = [
                mps_operation_from_gate_operation(op, self._qudit_to_index_map)
                for moment in self for op in moment]
else:
    class MPSimCircuit:  # type: ignore[no-redef]
        def __init__(self, *args, **kwargs):
            raise ImportError("MPSimCircuit needs cirq, which is not installed")
