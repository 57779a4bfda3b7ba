"""GB300-native matrix-product-state circuit simulator with mpsim's API.

Drop-in use: ``import mpsim_gb300 as mpsim`` then ``mpsim.MPS(...)``,
``mpsim.hgate()``, ``mpsim.MPSOperation(...)``; the Cirq front end is at
``mpsim_gb300.mpsim_cirq.simulator.MPSimulator`` as in the reference.
"""
from mpsim_gb300.core import MPS, MPSOperation, CannotConvertToMPSOperation
from mpsim_gb300.gates import (
    igate,
    xgate,
    ygate,
    zgate,
    hgate,
    rgate,
    cnot,
    cphase,
    swap,
)

__all__ = ["MPS", "MPSOperation", "CannotConvertToMPSOperation", "igate", "xgate", "ygate",
           "zgate", "hgate", "rgate", "cnot", "cphase", "swap"]
