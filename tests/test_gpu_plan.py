"""CircuitPlan: whole circuits (one or many) planned once, run eagerly or
replayed as one CUDA graph, against the gate-by-gate public API
(MPS.apply_layer) and the oracle.

The plan runs the same kernels on the same inputs as the public API, so its
states must agree with it to FP32 rounding (relative 1e-5 on amplitudes and
norms); a graph replay must reproduce the eager run bit for bit (its extra
sweeps find converged jobs and return at once).
"""
import numpy as np
import pytest
import torch

from mpsim_gb300 import _native
from mpsim_gb300 import circuits as C
from mpsim_gb300.core import MPS
from mpsim_gb300.plan import CircuitPlan

pytestmark = pytest.mark.gpu


def api_state(circ, precision="plain"):
    mps = MPS(circ.nqudits, circ.d, precision=precision)
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for lay in circ.layers:
        mps.apply_layer(lay.one_q, lay.pair_left, lay.two_q, **kw)
    return mps


def assert_same_state(a, b, rtol=1e-5):
    assert a.bond_dimensions() == b.bond_dimensions()
    wa, wb = a.wavefunction(), b.wavefunction()
    scale = max(np.max(np.abs(wb)), 1e-30)
    assert np.max(np.abs(wa - wb)) <= rtol * scale, np.max(np.abs(wa - wb)) / scale


def test_single_circuit_plan_matches_api(cuda):
    circ = C.brickwork(12, 8, d=2, maxsvals=16, seed=3)
    plan = CircuitPlan([circ])
    plan.run()
    plan.check_status()
    assert plan.n_two_qudit_gates == circ.n_two_qudit_gates
    assert_same_state(plan.state(0), api_state(circ))


def test_multi_circuit_plan_uneven_sizes(cuda):
    """Circuits of different qudit counts, depths and maxsvals, with CNOT/CZ
    slots (the mixed-batch workload's gate set), advanced together: each one
    equals its own run through the public API."""
    circs = [C.brickwork(10, 6, maxsvals=8, seed=1, instance=0, special_fraction=0.2),
             C.brickwork(14, 9, maxsvals=32, seed=1, instance=1, special_fraction=0.2),
             C.brickwork(8, 3, maxsvals=None, seed=1, instance=2, special_fraction=0.2),
             C.brickwork(12, 11, maxsvals=16, seed=1, instance=3, special_fraction=0.2)]
    plan = CircuitPlan(circs)
    plan.run()
    plan.check_status()
    for i, c in enumerate(circs):
        assert_same_state(plan.state(i), api_state(c))


def test_qutrit_plan(cuda):
    circs = [C.brickwork(7, 6, d=3, maxsvals=12, seed=4, instance=i) for i in range(3)]
    plan = CircuitPlan(circs)
    plan.run()
    for i, c in enumerate(circs):
        assert_same_state(plan.state(i), api_state(c))


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_graph_replay_equals_eager(cuda, precision):
    """The whole circuit captured as one CUDA graph (the two-qudit calls read
    nothing back under capture): two replays give the eager run's state bit
    for bit, and the status words report nothing."""
    circs = [C.brickwork(16, 10, maxsvals=64, seed=9, instance=i) for i in range(2)]
    plan = CircuitPlan(circs, precision=precision)
    plan.run()
    torch.cuda.synchronize()
    eager = [[t.clone() for t in plan.final_sites(i)] for i in range(len(circs))]
    plan.capture()
    for _ in range(2):
        for i in range(len(circs)):
            for t in plan.final_sites(i):
                t.zero_()
        plan.replay()
        torch.cuda.synchronize()
        for i in range(len(circs)):
            for t, e in zip(plan.final_sites(i), eager[i]):
                assert torch.equal(t, e)
    assert_same_state(plan.state(0), api_state(circs[0], precision))


def test_mixed_plan_against_dense_fp64(cuda):
    """precision="mixed" in a plan whose middle gates reach 128 columns,
    against the dense complex128 evolution: infidelity <= 1e-5."""
    from oracle.dense import DenseState
    circ = C.brickwork(14, 10, maxsvals=None, seed=11)
    plan = CircuitPlan([circ], precision="mixed")
    plan.run()
    st = DenseState(14, 2)
    for lay in circ.layers:
        for i in range(14):
            st.apply_one(lay.one_q[i], i)
        for p, i in enumerate(lay.pair_left):
            st.apply_two(lay.two_q[p], int(i), int(i) + 1)
    ref = st.vector()
    got = plan.state(0).wavefunction().astype(np.complex128)
    infid = 1 - abs(np.vdot(ref, got)) ** 2 / (np.vdot(ref, ref).real * np.vdot(got, got).real)
    assert infid <= 1e-5, infid


def test_status_words_report_unconverged(cuda):
    """A sweep cap of 1 leaves the chi=32 gates unconverged: under capture the
    call cannot return an error, so replay() raises from the status words."""
    circ = C.brickwork(12, 8, maxsvals=32, seed=2)
    CircuitPlan([circ]).run()            # per-device set-up of every kernel, outside capture
    plan = CircuitPlan([circ], max_sweeps=1)
    with pytest.raises(_native.NativeError):
        plan.run()                       # eager: the call itself reports
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run()
    plan.graph = g
    with pytest.raises(_native.NativeError) as ei:
        plan.replay()
    assert ei.value.code == _native.MPS_ERR_NOT_CONVERGED
