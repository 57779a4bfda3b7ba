"""The batched workloads at their own sizes, against the oracle: a seeded
subsample of the 512-circuit mixed batch (16-48 qubits, maxsvals 16-128, with
its CNOT/CZ slots) and a prefix of a 32-qutrit, maxsvals=192 circuit (theta up
to 576 x 576), through the batched form (CircuitPlan) and the public API.

Checks (gauge-invariant; the tolerances of test_gpu_circuit_parity.py):
exact kept counts and bond dimensions; per-gate singular values within 2e-5
of s_0 until a gate discards more than 1e-3 of its weight, afterwards against
the oracle's own complex64-vs-complex128 spread (median ratio <= 20, every
gate within 100x + 1e-4); the final norm within 10x that spread (at least
1e-3 relative); and, where no cut is near-degenerate, the final state's
infidelity against the complex128 oracle within 20x the complex64 oracle's.
A cut with s_(k-1) - s_k < 1e-4 s_0 (CNOT and CZ on product-like states make
exact ties) leaves the kept vectors arbitrary for any SVD, so comparisons
stop at the first such gate and only its kept weight is checked.
"""
import numpy as np
import pytest
import torch

from mpsim_gb300 import circuits as C
from mpsim_gb300.core import MPS
from mpsim_gb300.plan import CircuitPlan
from oracle.ref_mps import OracleMPS, overlap_infidelity
from test_gpu_circuit_parity import _chaotic_checks

pytestmark = pytest.mark.gpu


def oracle_run(circ, dtype):
    o = OracleMPS(circ.nqudits, circ.d, dtype)
    o.record = True
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for lay in circ.layers:
        for q in range(circ.nqudits):
            o.apply_one_qudit_gate(lay.one_q[q], q)
        for p, j in enumerate(lay.pair_left):
            o.apply_two_qudit_gate(lay.two_q[p], int(j), int(j) + 1, **kw)
    return o


def gpu_run(circ, precision="plain"):
    mps = MPS(circ.nqudits, circ.d, record_svals=True, precision=precision)
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for lay in circ.layers:
        mps.apply_layer(lay.one_q, lay.pair_left, lay.two_q, **kw)
    torch.cuda.synchronize()
    return mps


def as_oracle(mps):
    o = OracleMPS(mps.nqudits, mps.qudit_dimension, np.complex128)
    o.sites = [t.detach().cpu().numpy().astype(np.complex128) for t in mps.sites]
    return o


def prefix(circ, nlayers):
    c = C.BrickworkCircuit(circ.nqudits, circ.d, nlayers, circ.maxsvals, circ.seed,
                           circ.instance)
    c.layers = circ.layers[:nlayers]
    return c


def compare(circ, mps, tag):
    o128, o64 = oracle_run(circ, np.complex128), oracle_run(circ, np.complex64)
    assert list(mps.bond_dimensions()) == o128.bond_dimensions(), tag
    errs, spreads, stop = [], [], len(o128.history)
    for g, ((s, k, _), (r, kr, _), (r64, _, _)) in enumerate(
            zip(mps.svals_history, o128.history, o64.history)):
        assert k == kr, (tag, g)
        if 0 < k < len(r) and r[k - 1] - r[k] < 1e-4 * r[0]:
            # near-degenerate cut: only the kept weight is determined
            assert abs(np.sum(s[:k] ** 2) - np.sum(r[:k] ** 2)) <= 1e-4 * np.sum(r ** 2), (tag, g)
            stop = g
            break
        errs.append(np.max(np.abs(s[:k] - r[:k])) / r[0] if k else 0.0)
        spreads.append(np.max(np.abs(r64[:k] - r[:k])) / r[0] if k else 0.0)
    n128, n64 = o128.norm(), o64.norm()
    disc = np.array([h[2] for h in o128.history[:stop]])
    pre = int(np.argmax(disc > 1e-3)) if np.any(disc > 1e-3) else len(disc)
    _chaotic_checks(errs, spreads, pre, tag)
    if stop == len(o128.history):
        assert abs(mps.norm() - n128) / n128 < max(10 * abs(n64 - n128) / n128, 1e-3), tag
        inf = overlap_infidelity(as_oracle(mps), o128)
        inf64 = overlap_infidelity(o64, o128)
        assert inf <= max(20 * inf64, 1e-6), (tag, inf, inf64)
    return stop, n128, n64


def test_mixed_batch_subsample_with_cnot_cz(cuda):
    """The two cheapest circuits of each maxsvals class (16, 32, 64, 128) among
    the first 48 of the 512-circuit batch (its seeds), all with CNOT/CZ
    slots, run through the batched plan: each equals its gate-by-gate run,
    which matches the oracle as above."""
    every = C.mixed_batch(48, seed=0)
    order = []
    for chi in (16, 32, 64, 128):
        cls = [i for i in range(len(every)) if every[i].maxsvals == chi]
        order += sorted(cls, key=lambda i: C.estimated_cost(every[i]))[:2]
    circs = [every[i] for i in order]
    assert all(any((np.abs(np.abs(l.two_q) - np.abs(l.two_q).round()) < 1e-12).all(axis=(1, 2)).any()
                   for l in c.layers) for c in circs)          # a CNOT or CZ in every circuit
    plan = CircuitPlan(circs)
    plan.run()
    plan.check_status()
    full = 0
    for i, c in enumerate(circs):
        mps = gpu_run(c)
        stop, n128, n64 = compare(c, mps, f"batch circuit {order[i]}")
        full += stop == c.n_two_qudit_gates
        # the batched form's state against the gate-by-gate one (different
        # call groupings round differently; the truncated dynamics amplifies
        # that like any other rounding)
        ps = plan.state(i)
        assert ps.bond_dimensions() == mps.bond_dimensions()
        assert abs(ps.norm() - mps.norm()) <= max(10 * abs(n64 - n128), 1e-3 * n128)
    assert full >= 4, "too many near-degenerate cuts: the subsample checks too little"


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_qutrit_chi192_prefix(cuda, precision):
    """The first 10 layers of a 32-qutrit, maxsvals=192 circuit of the qutrit
    batch: bonds reach 192 and theta 576 x 576 from layer 6, and the later
    gates discard weight."""
    circ = prefix(C.qutrit_batch(1, seed=0, workers=1)[0], 10)
    mps = gpu_run(circ, precision)
    assert max(mps.bond_dimensions()) == 192
    compare(circ, mps, f"qutrit prefix ({precision})")
