"""Deferred two-qudit gates: apply_two_qudit_gate queues gates on disjoint
adjacent pairs and runs them as one batched launch when a later gate shares
a site or any operation reads the sites.  The results must equal applying the
gates one by one (exactly: the same kernels run on the same inputs)."""
import numpy as np
import pytest

from mpsim_gb300 import MPS, MPSOperation
from mpsim_gb300 import circuits as C
from mpsim_gb300 import gates as G

pytestmark = pytest.mark.gpu


def gate_by_gate(circ, timing=None):
    m = MPS(circ.nqudits, circ.d)
    m.timing = timing
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for kind, sites, mat in circ.operations():
        if kind == 1:
            m.apply_one_qudit_gate(np.asarray(mat), sites[0])
        else:
            m.apply_two_qudit_gate(np.asarray(mat).reshape((circ.d,) * 4), sites[0], sites[1], **kw)
    return m


def by_layer(circ):
    m = MPS(circ.nqudits, circ.d)
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for lay in circ.layers:
        m.apply_layer(lay.one_q, lay.pair_left, lay.two_q, **kw)
    return m


def test_gate_by_gate_is_batched_and_exact(cuda):
    circ = C.brickwork(12, 8, d=2, maxsvals=16, seed=4)
    timing = []
    a = gate_by_gate(circ, timing)
    b = by_layer(circ)
    assert np.allclose(a.wavefunction(), b.wavefunction(), atol=1e-5)
    assert list(a.bond_dimensions()) == list(b.bond_dimensions())
    # one batched call per layer, not one per gate
    assert len(timing) <= circ.depth + 1
    assert sum(t[0] for t in timing) == circ.n_two_qudit_gates


def test_reads_flush_queued_gates(cuda):
    m = MPS(4)
    m.h(0)
    m.h(2)
    m.cnot(0, 1)
    m.cnot(2, 3)                       # both queued, disjoint
    assert m._pending and len(m._pending) == 2
    assert list(m.bond_dimensions()) == [2, 1, 2]
    assert not m._pending
    m.cnot(1, 2)
    assert abs(m.norm() - 1.0) < 1e-6  # norm flushes
    m.cnot(1, 2)
    c = m.copy()                       # copy flushes and starts with an empty queue
    assert not m._pending and not c._pending
    assert np.allclose(c.wavefunction(), m.wavefunction())
    m.cnot(0, 1)
    rho = m.reduced_density_matrix([0])
    assert np.allclose(np.trace(rho), 1.0, atol=1e-6)


def test_one_qudit_gate_on_queued_site_waits(cuda):
    # x then cnot on (0,1) queued, then h on 1: h must act after the cnot
    a = MPS(3)
    a.x(0)
    a.cnot(0, 1)
    a.h(1)
    psi = a.wavefunction()
    ref = np.zeros(8, np.complex128)
    ref[0b100] = 1 / np.sqrt(2)
    ref[0b110] = -1 / np.sqrt(2)
    assert np.allclose(psi, ref, atol=1e-6)


def test_apply_operations_and_nonadjacent(cuda):
    circ = C.brickwork(8, 5, d=2, maxsvals=None, seed=9)
    ops = [MPSOperation(G.Node(np.asarray(mat).reshape((2,) * (2 * kind))), sites)
           for kind, sites, mat in circ.operations()]
    a = MPS(8)
    a.apply(ops)
    b = by_layer(circ)
    assert np.allclose(a.wavefunction(), b.wavefunction(), atol=1e-5)
    # non-adjacent gates run their swap chains in order behind queued gates
    m = MPS(5)
    m.h(0)
    for i in range(1, 5):
        m.cnot(0, i)
    psi = m.wavefunction()
    assert abs(abs(psi[0]) - 2 ** -0.5) < 1e-6 and abs(abs(psi[-1]) - 2 ** -0.5) < 1e-6


def test_one_qudit_gates_are_queued_and_ordered(cuda):
    rng = np.random.default_rng(3)
    u = [G.haar_random_matrix(1, 2, 40 + i) for i in range(6)]
    w, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
    a = MPS(6)
    for i in range(6):
        a.apply_one_qudit_gate(u[i], i)
    assert len(a._pending_1q) == 6            # one launch for all six
    mine = w.copy()
    a.apply_one_qudit_gate(mine, 5)            # site 5 is queued: the six run first
    assert len(a._pending_1q) == 1
    mine[:] = 0                                # reusing the array must not change the queued gate
    a.cnot(2, 3)                               # queued beside the gate on 5
    a.apply_one_qudit_gate(u[0], 2)            # site 2 waits for the cnot
    psi = a.wavefunction()
    state = np.zeros(2 ** 6, complex)
    state[0] = 1
    state = state.reshape((2,) * 6)

    def one(st, g, q):
        return np.moveaxis(np.tensordot(g, st, axes=([1], [q])), 0, q)
    for i in range(6):
        state = one(state, u[i], i)
    state = one(state, w, 5)
    cn = np.asarray(G.cnot().tensor).reshape(2, 2, 2, 2)
    state = np.moveaxis(np.tensordot(cn, state, axes=([2, 3], [2, 3])), [0, 1], [2, 3])
    state = one(state, u[0], 2)
    assert np.allclose(psi, state.reshape(-1), atol=2e-6)


def test_disjoint_swap_chains_are_interleaved(cuda, monkeypatch):
    """MPS.apply interleaves the SWAP chains of two-qudit operations on
    disjoint site ranges (the k-th SWAP of each chain in one launch): the
    state equals in-order application (apply_two_qudit_gate one by one, with
    truncating SWAPs) with fewer launches, and without truncation the oracle's
    state; overlapping ranges stay in order."""
    from oracle.ref_mps import OracleMPS
    n, d = 12, 2
    rng = np.random.default_rng(21)
    ops = []
    for layer in range(4):
        for q in range(n):
            u1 = G.haar_random_matrix(1, 2, int(rng.integers(1 << 30)))
            ops.append(MPSOperation(G.Node(np.asarray(u1)), q))
        # disjoint long-range pairs (both orientations) and an adjacent one,
        # then one whose range overlaps them
        for a, b in ((0, 4), (9, 5), (10, 11), (3, 8)):
            u = G.haar_random_matrix(2, 2, int(rng.integers(1 << 30)))
            ops.append(MPSOperation(G.Node(np.asarray(u).reshape((2,) * 4)), (a, b)))

    calls = []
    orig = MPS._run_pair_group
    monkeypatch.setattr(MPS, "_run_pair_group",
                        lambda self, pairs, prec: (calls.append(len(pairs)), orig(self, pairs, prec)))

    def in_order(kw):
        m = MPS(n, d)
        for op in ops:
            if op.is_single_qudit_operation():
                m.apply_one_qudit_gate(op.node(), op.qudit_indices[0])
            else:
                m.apply_two_qudit_gate(op.node(), *op.qudit_indices, **kw)
                m._flush()
        return m

    kw = {"maxsvals": 6}
    a = MPS(n, d)
    a.apply(ops, **kw)
    wa = a.wavefunction()
    inter = list(calls)
    calls.clear()
    b = in_order(kw)
    wb = b.wavefunction()
    seq = list(calls)
    assert list(a.bond_dimensions()) == list(b.bond_dimensions())
    assert np.allclose(wa, wb, atol=1e-5)
    assert sum(inter) == sum(seq)            # the same gates ...
    assert len(inter) < len(seq)             # ... in fewer launches
    assert max(inter) >= 3                   # the disjoint chains shared launches

    a = MPS(n, d)
    a.apply(ops)
    o = OracleMPS(n, d)
    for op in ops:
        if op.is_single_qudit_operation():
            o.apply_one_qudit_gate(np.asarray(op.tensor()), op.qudit_indices[0])
        else:
            o.apply_two_qudit_gate(np.asarray(op.tensor()), *op.qudit_indices)
    assert np.allclose(a.wavefunction(), o.wavefunction(), atol=2e-6)
    assert list(a.bond_dimensions()) == [int(s.shape[2]) for s in o.sites[:-1]]
