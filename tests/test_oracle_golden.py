"""The NumPy oracle against the reference's own outputs (CPU).

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py,
which executes the reference's unmodified mpsim/core.py (through a
restatement of the TensorNetwork 0.2.1 calls it makes) on seeded circuits.
"""
import os

import numpy as np
import pytest

from oracle.dense import DenseState
from oracle.ref_mps import OracleMPS, canonical_spectra, overlap_infidelity
from mpsim_gb300 import circuits as C
from mpsim_gb300 import gates as G

from conftest import GOLDEN


def run_oracle(circ, dtype, upto_layer=None):
    o = OracleMPS(circ.nqudits, circ.d, dtype)
    o.record = True
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for t, lay in enumerate(circ.layers):
        if upto_layer is not None and t >= upto_layer:
            break
        for i in range(circ.nqudits):
            o.apply_one_qudit_gate(lay.one_q[i], i)
        for p, i in enumerate(lay.pair_left):
            o.apply_two_qudit_gate(lay.two_q[p], int(i), int(i) + 1, **kw)
    return o


def spectra(z, prefix):
    v, off = z[prefix + "_svals"], z[prefix + "_offsets"]
    return [v[off[g]:off[g + 1]] for g in range(len(off) - 1)]


def sval_err(a, b):
    """max |a-b| / (1e-5 b + 1e-6 b_0): <= 1 means within tolerance."""
    k = min(len(a), len(b))
    return float(np.max(np.abs(a[:k] - b[:k]) / (1e-5 * b[:k] + 1e-6 * b[0])))


def test_reference_unit_tests_pass_under_shim():
    with open(os.path.join(GOLDEN, "reference_tests_under_shim.txt")) as f:
        lines = [l for l in f if not l.startswith("#")]
    assert len(lines) >= 140
    assert all(l.startswith("PASSED") for l in lines), [l for l in lines if not l.startswith("PASSED")]


@pytest.mark.parametrize("name", ["brickwork_10q_d10_full", "brickwork_8qutrit_d8_chi12"])
@pytest.mark.parametrize("tag,dtype", [("c64", np.complex64), ("c128", np.complex128)])
def test_oracle_matches_reference_small(name, tag, dtype):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    circ = C.workload(name) if name in C.WORKLOADS else C.brickwork(8, 8, d=3, maxsvals=12, seed=3)
    o = run_oracle(circ, dtype)
    ref = spectra(z, f"ref_{tag}")
    assert len(ref) == len(o.history)
    tol = 3.0 if tag == "c64" else 1e-6
    for g, (s, k, _) in enumerate(o.history):
        assert k == z[f"ref_{tag}_kept"][g]
        assert sval_err(s, ref[g]) < tol, g
    amp = o.amplitudes(z["bitstrings"])
    ra = z[f"ref_{tag}_amplitudes"]
    rel = np.linalg.norm(amp - ra) / np.linalg.norm(ra)
    assert rel < (1e-5 if tag == "c64" else 1e-12)
    if f"ref_{tag}_wavefunction" in z:
        wf = o.wavefunction()
        assert np.allclose(wf, z[f"ref_{tag}_wavefunction"], atol=1e-6 if tag == "c64" else 1e-13)
    assert np.isclose(o.norm(), z[f"ref_{tag}_norms"][-1], rtol=1e-5)


def test_oracle_matches_reference_48q_prefix():
    """48 qubits, maxsvals=128: the first 12 layers (before the truncated
    dynamics amplifies rounding) agree with the reference run in complex128."""
    z = np.load(os.path.join(GOLDEN, "brickwork_48q_d24_chi128.npz"))
    circ = C.workload("brickwork_48q_d24_chi128")
    o = run_oracle(circ, np.complex128, upto_layer=12)
    ref = spectra(z, "ref_c128")
    for g, (s, k, _) in enumerate(o.history):
        assert k == z["ref_c128_kept"][g]
        assert sval_err(s, ref[g]) < 1e-3, g
    assert np.isclose(o.norm(), z["ref_c128_norms"][len(o.history) - 1], rtol=1e-9)


def test_reference_fixture_self_consistency_48q():
    """Full 24 layers: the reference's bond dimensions and kept counts match
    the oracle's fixture, and its c64 and c128 runs end within 1e-3 in norm."""
    z = np.load(os.path.join(GOLDEN, "brickwork_48q_d24_chi128.npz"))
    assert (z["ref_c64_kept"] == z["oracle_c64_kept"]).all()
    assert (z["ref_c128_kept"] == z["oracle_c128_kept"]).all()
    n64, n128 = z["ref_c64_norms"][-1], z["ref_c128_norms"][-1]
    assert abs(n64 - n128) / n128 < 1e-3
    ref = spectra(z, "ref_c128")
    orc = spectra(z, "oracle_c128")
    assert max(sval_err(a, b) for a, b in zip(orc, ref)) < 50.0


def test_known_answers_against_reference_fixture():
    z = np.load(os.path.join(GOLDEN, "known_answers.npz"))
    # Bell with maxsvals=1
    o = OracleMPS(2, 2, np.complex128)
    o.apply_one_qudit_gate(G.hgate().tensor, 0)
    o.apply_two_qudit_gate(G.cnot().tensor, 0, 1, maxsvals=1)
    assert np.allclose(o.wavefunction(), z["bell_maxsvals1"])
    assert np.allclose(z["bell_maxsvals1"], [2 ** -0.5, 0, 0, 0])
    # GHZ with non-local CNOTs
    o = OracleMPS(5, 2, np.complex128)
    o.apply_one_qudit_gate(G.hgate().tensor, 0)
    for i in range(1, 5):
        o.apply_two_qudit_gate(G.cnot().tensor, 0, i)
    assert np.allclose(o.wavefunction(), z["ghz5_nonlocal"])
    # QFT
    o = OracleMPS(4, 2, np.complex128)
    for i in range(3, -1, -1):
        o.apply_one_qudit_gate(G.hgate().tensor, i)
        for j in range(i - 1, -1, -1):
            o.apply_two_qudit_gate(G.cphase(2 ** (j - i)).tensor, j, i)
    assert np.allclose(o.wavefunction(), z["qft4"])
    assert np.allclose(z["qft4"], np.ones(16) / 4)
    o = OracleMPS(2, 2, np.complex128)
    o.apply_one_qudit_gate(G.hgate().tensor, 0)
    o.apply_two_qudit_gate(G.cnot().tensor, 0, 1, fraction=0.5)
    assert np.allclose(o.wavefunction(), z["bell_fraction_half"])
    # qutrits, mixed canonical forms, flipped pair
    o = OracleMPS(4, 3, np.complex128)
    for i in range(4):
        o.apply_one_qudit_gate(C.haar_random_matrix(1, 3, 11 + i), i)
    for (a, b) in [(0, 1), (2, 3), (1, 2), (2, 1), (0, 1)]:
        g = C.haar_random_matrix(2, 3, 100 + a * 7 + b)
        o.apply_two_qudit_gate(g, a, b, keep_left_canonical=(a != 2))
    assert np.allclose(o.wavefunction(), z["qutrit4_mixed"])


def test_oracle_untruncated_equals_dense():
    circ = C.brickwork(7, 6, d=2, seed=11)
    o = run_oracle(circ, np.complex128)
    ds = DenseState(7, 2)
    for kind, sites, mat in circ.operations():
        if kind == 1:
            ds.apply_one(mat, sites[0])
        else:
            ds.apply_two(mat, sites[0], sites[1])
    assert np.allclose(o.wavefunction(), ds.vector(), atol=1e-12)


def test_oracle_nonadjacent_and_flipped_equal_dense():
    rng = np.random.default_rng(3)
    o = OracleMPS(6, 2, np.complex128)
    ds = DenseState(6, 2)
    for step in range(12):
        i, j = rng.choice(6, 2, replace=False)
        g = C.haar_random_matrix(2, 2, 1000 + step)
        o.apply_two_qudit_gate(g, int(i), int(j))
        ds.apply_two(g, int(i), int(j))
    assert np.allclose(o.wavefunction(), ds.vector(), atol=1e-12)


def test_canonical_spectra_gauge_invariant():
    circ = C.brickwork(8, 5, d=2, maxsvals=6, seed=2)
    a = run_oracle(circ, np.complex128)
    b = a.copy()
    # random invertible gauge on bond 3 leaves the state and its spectra unchanged
    rng = np.random.default_rng(0)
    chi = b.sites[3].shape[2]
    x = rng.normal(size=(chi, chi)) + 1j * rng.normal(size=(chi, chi))
    b.sites[3] = np.tensordot(b.sites[3], x, axes=([2], [0]))
    b.sites[4] = np.tensordot(np.linalg.inv(x), b.sites[4], axes=([1], [0]))
    assert overlap_infidelity(a, b) < 1e-12
    for s, t in zip(canonical_spectra(a), canonical_spectra(b)):
        assert np.allclose(s, t, atol=1e-10)
