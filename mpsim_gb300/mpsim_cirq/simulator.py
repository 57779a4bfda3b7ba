"""MPSimulator with mpsim's interface (mpsim/mpsim_cirq/simulator.py:14-88).

``MPSimulator(options)`` forwards ``options`` (``maxsvals``, ``fraction``,
``keep_left_canonical`` ...) to ``MPS.apply`` exactly as the reference does.
It simulates Cirq circuits when Cirq is installed, and also accepts, without
Cirq, a sequence of ``MPSOperation`` (the qudit count is the largest index
plus one) or a seeded ``circuits.BrickworkCircuit``.
"""
from __future__ import annotations

from typing import Any, List

import numpy as np

from mpsim_gb300.core import MPS, MPSOperation
from mpsim_gb300.gates import Node
from mpsim_gb300.mpsim_cirq.circuits import cirq, mps_operation_from_gate_operation


class MPSimulator:
    def __init__(self, options: dict = {}):
        self._options = options

    def simulate(self, program, param_resolver=None, qubit_order=None, initial_state=None):
        params = param_resolver if param_resolver is not None else None
        return self.simulate_sweep(program, params, qubit_order, initial_state)[0]

    def simulate_sweep(self, program, params=None, qubit_order=None,
                       initial_state: Any = None) -> List[MPS]:
        if cirq is not None and isinstance(program, cirq.Circuit):  # pragma: no cover
            resolvers = cirq.study.to_resolvers(params)
            out = []
            for prs in resolvers:
                solved = cirq.protocols.resolve_parameters(program, prs)
                order = cirq.ops.QubitOrder.as_qubit_order(
                    qubit_order if qubit_order is not None else cirq.ops.QubitOrder.DEFAULT
                ).order_for(solved.all_qubits())
                index = {q: i for i, q in enumerate(order)}
                mps = MPS(nqudits=len(solved.all_qubits()))
                ops = [mps_operation_from_gate_operation(op, index)
                       for op in solved.all_operations()]
                mps.apply(ops, **self._options)
                out.append(mps)
            return out
        if hasattr(program, "layers") and hasattr(program, "nqudits"):
            mps = MPS(program.nqudits, program.d)
            opts = dict(self._options)
            if program.maxsvals is not None and "maxsvals" not in opts and "fraction" not in opts:
                opts["maxsvals"] = program.maxsvals
            for lay in program.layers:
                mps.apply_layer(lay.one_q, lay.pair_left, lay.two_q, **opts)
            return [mps]
        try:
            ops = list(program)
        except TypeError:
            raise ValueError(
                f"Program is of type {type(program)} but should be either a cirq.Circuit, an "
                "mpsim_gb300 circuit or a sequence of MPSOperation.")
        if not ops or not all(isinstance(o, MPSOperation) for o in ops):
            raise ValueError("Program must be a non-empty sequence of MPSOperation.")
        n = 1 + max(max(o.qudit_indices) for o in ops)
        d = ops[0].qudit_dimension
        mps = MPS(nqudits=n, qudit_dimension=d)
        mps.apply(ops, **self._options)
        return [mps]
