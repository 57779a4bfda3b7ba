"""The multi-circuit form (mpsim_gb300.batch) against single-circuit runs
and the complex128 oracle: circuits of different sizes, depths and
truncations advanced together must each end where they would alone.
Tolerances: infidelity < 1e-9 against the single-circuit GPU run and
< 1e-8 against the oracle (these circuits are small enough not to amplify
rounding), identical bond dimensions."""
import numpy as np
import pytest
import torch

from mpsim_gb300 import circuits as C
from mpsim_gb300.batch import MPSBatch, run_circuits
from mpsim_gb300.core import MPS
from oracle.ref_mps import OracleMPS

pytestmark = pytest.mark.gpu


def _infid(a, b):
    a, b = a.astype(np.complex128), b.astype(np.complex128)
    return 1.0 - abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)


def _alone(circ):
    m = MPS(circ.nqudits, circ.d)
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for lay in circ.layers:
        m.apply_layer(lay.one_q, lay.pair_left, lay.two_q, **kw)
    return m


def _oracle(circ):
    o = OracleMPS(circ.nqudits, circ.d, np.complex128)
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for kind, sites, mat in circ.operations():
        if kind == 1:
            o.apply_one_qudit_gate(mat, sites[0])
        else:
            o.apply_two_qudit_gate(mat, *sites, **kw)
    return o


@pytest.mark.parametrize("d", [2, 3])
def test_batch_matches_single_runs(cuda, d):
    specs = [(6, 4, 4), (9, 7, 8), (11, 10, None), (8, 3, 2), (12, 9, 16)] if d == 2 else \
            [(5, 4, 6), (7, 6, 9), (8, 5, None)]
    # Haar gates only: fixed CNOT/CZ gates make exactly degenerate singular
    # values, where which vectors a truncation keeps is decided by rounding
    circs = [C.brickwork(n, depth, d=d, maxsvals=chi, seed=17, instance=i)
             for i, (n, depth, chi) in enumerate(specs)]
    states = run_circuits(circs)
    torch.cuda.synchronize()
    for circ, st in zip(circs, states):
        alone = _alone(circ)
        ora = _oracle(circ)
        assert st.bond_dimensions() == alone.bond_dimensions() == ora.bond_dimensions()
        wf = st.wavefunction()
        assert _infid(wf, alone.wavefunction()) < 1e-9
        assert _infid(wf, ora.wavefunction()) < 1e-8
        assert abs(st.norm() - ora.norm()) < 1e-5


def test_batch_rejects_bad_layers(cuda):
    states = [MPS(4), MPS(5)]
    b = MPSBatch(states)
    with pytest.raises(ValueError):
        b.step([(None, [0, 1], np.zeros((2, 4, 4))), None], [None, None])
    with pytest.raises(ValueError):
        MPSBatch([MPS(3, 2), MPS(3, 3)])
