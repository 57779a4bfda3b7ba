"""Host-side logic that needs no GPU: truncation parsing, bond bounds,
operation validity, gate library, seeded workloads, the C ABI's exports."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from mpsim_gb300 import MPSOperation, circuits as C, gates as G
from mpsim_gb300.core import MPS, kept_count, max_bond_dimensions, parse_truncation
from oracle import ref_mps

from conftest import REPO


def test_kept_count_follows_tensornetwork_slicing():
    assert kept_count(None, 7) == 7
    assert kept_count(3, 7) == 3
    assert kept_count(10, 7) == 7
    assert kept_count(0, 7) == 0
    assert kept_count(-1, 7) == 6          # s[:-1]
    assert kept_count(-10, 7) == 0
    for m in (None, 0, 1, 5, 9, -2):
        for r in range(0, 6):
            assert kept_count(m, r) == ref_mps.kept_count(m, r)


def test_parse_truncation_matches_reference_rules():
    mb = [2, 4, 8, 4, 2].__getitem__
    assert parse_truncation({}, mb, 0) is None
    assert parse_truncation({"maxsvals": 3}, mb, 0) == 3
    assert parse_truncation({"maxsvals": "5"}, mb, 0) == 5
    assert parse_truncation({"fraction": 0.5}, mb, 2) == 4
    assert parse_truncation({"fraction": 0.5}, mb, 0) == 1
    assert parse_truncation({"fraction": 0.25}, mb, 0) == 0   # round(0.5) == 0
    assert parse_truncation({"fraction": 0.75}, mb, 0) == 2   # round(1.5) == 2
    assert parse_truncation({"fraction": 1}, mb, 1) == 4
    with pytest.raises(ValueError):
        parse_truncation({"fraction": 0.5, "maxsvals": 1}, mb, 0)
    with pytest.raises(ValueError):
        parse_truncation({"fraction": 1.5}, mb, 0)
    with pytest.raises(TypeError):
        parse_truncation({"maxsvals": None}, mb, 0)


def test_max_bond_dimensions():                      # core_test.py:86-155
    assert max_bond_dimensions(5, 2) == [2, 4, 4, 2]
    assert max_bond_dimensions(7, 2) == [2, 4, 8, 8, 4, 2]
    assert max_bond_dimensions(6, 2) == [2, 4, 8, 4, 2]
    assert max_bond_dimensions(8, 2) == [2, 4, 8, 16, 8, 4, 2]
    assert max_bond_dimensions(5, 4) == [4, 16, 16, 4]
    assert max_bond_dimensions(4, 10) == [10, 100, 10]
    assert max_bond_dimensions(6, 10) == [10, 100, 1000, 100, 10]
    for n in range(2, 12):
        for d in (2, 3):
            assert max_bond_dimensions(n, d) == ref_mps.OracleMPS(n, d).max_bond_dimensions


def test_mps_needs_two_qudits():                     # core_test.py:71-75
    for d in (2, 3, 10, 100):
        with pytest.raises(ValueError):
            MPS(nqudits=1, qudit_dimension=d)


def test_mps_without_cuda_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        MPS(3)


def test_mps_operation():                            # core_test.py:25-68
    op = MPSOperation(G.igate(), qudit_indices=0, qudit_dimension=2)
    assert op.qudit_indices == (0,) and op.qudit_dimension == 2
    assert op.is_valid() and op.is_unitary()
    assert op.is_single_qudit_operation() and not op.is_two_qudit_operation()
    rng = np.random.RandomState(1)
    t = rng.randn(2, 2)
    op = MPSOperation(G.Node(t), qudit_indices=(0,))
    assert np.allclose(op.tensor(), t)
    assert op.node(copy=True).tensor is not t
    op = MPSOperation(G.cnot(), (0, 2))
    assert op.is_valid() and op.is_two_qudit_operation()
    assert not MPSOperation(G.cnot(), (0,)).is_valid()
    assert not MPSOperation(G.hgate(), (0,), qudit_dimension=3).is_valid()


def test_gate_library():                             # gates_test.py:21-83, gates.py dtypes
    for g in (G.igate(), G.hgate(), G.xgate(), G.ygate(), G.zgate(), G.cnot()):
        assert G.is_unitary(g)
    for e in np.linspace(0, 2 * np.pi, 20):
        assert G.is_unitary(G.cphase(e))
    assert G.cnot().tensor.dtype == np.float64 and G.swap().tensor.dtype == np.float64
    assert G.hgate().tensor.dtype == np.complex64
    p0 = G.computational_basis_projector(0)
    assert np.array_equal(p0.tensor, [[1, 0], [0, 0]]) and G.is_projector(p0)
    assert not G.is_unitary(p0) and str(p0) == "|0><0|"
    with pytest.raises(ValueError):
        G.computational_basis_projector(-1)
    with pytest.raises(ValueError):
        G.computational_basis_projector(10, dim=8)
    for n in (1, 2, 3):
        for d in (2, 3, 5):
            h = G.haar_random_unitary(n, d, seed=1)
            assert h.tensor.dtype == np.complex128 and h.tensor.shape == (d,) * (2 * n)
            assert G.is_unitary(h)
            # identical to the oracle's restatement of gates.py:248-286
            assert np.array_equal(h.tensor, ref_mps.haar_random_unitary(n, d, seed=1))


def test_workloads_are_seeded_and_sized():
    c0 = C.workload("brickwork_10q_d10_full")
    assert c0.n_two_qudit_gates == 45 and c0.maxsvals is None
    assert C.workload("brickwork_48q_d24_chi128").n_two_qudit_gates == 564
    c2 = C.workload("brickwork_64q_d40_chi256")
    assert c2.n_two_qudit_gates == 1260 and c2.maxsvals == 256
    again = C.workload("brickwork_10q_d10_full")
    for a, b in zip(c0.layers, again.layers):
        assert np.array_equal(a.one_q, b.one_q) and np.array_equal(a.two_q, b.two_q)
    other = C.workload("brickwork_10q_d10_full", instance=1)
    assert not np.array_equal(other.layers[0].two_q, c0.layers[0].two_q)
    for lay in c0.layers:
        for u in list(lay.one_q) + list(lay.two_q):
            assert np.allclose(u.conj().T @ u, np.eye(u.shape[0]), atol=1e-12)
    batch = C.mixed_batch(16)
    for c in batch:
        assert 16 <= c.nqudits <= 48 and 8 <= c.depth <= 32 and c.maxsvals in (16, 32, 64, 128)
    q = C.qutrit_batch(2)
    assert q[0].d == 3 and q[0].nqudits == 32 and q[0].layers[0].two_q.shape[1:] == (9, 9)


def _header_symbols():
    with open(os.path.join(REPO, "include", "mpsim_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(mps_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_header_symbol(built_lib):
    from mpsim_gb300 import _native
    syms = _header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(built_lib, s), s
        assert s in _native.SIGNATURES, s
    assert built_lib.mps_version() >= 100
    assert built_lib.mps_2q_workspace_bytes(0, 4, 4, 2) == 0
    assert built_lib.mps_2q_workspace_bytes(32, 512, 512, 2) >= 32 * 2 * 512 * 512 * 8
    # the mixed form adds three bf16 piece planes (12 bytes a complex element)
    assert (built_lib.mps_2q_workspace_bytes_mixed(32, 512, 512, 2)
            >= built_lib.mps_2q_workspace_bytes(32, 512, 512, 2) + 32 * 512 * 512 * 12)
    assert built_lib.mps_2q_workspace_bytes_mixed(0, 4, 4, 2) == 0


def test_job_struct_layout_matches_header(tmp_path):
    """The ctypes/numpy mirror of mps_2q_job has the C layout."""
    from mpsim_gb300 import _native
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "mpsim_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(mps_2q_job),"
        " offsetof(mps_2q_job, status), offsetof(mps_2q_job, chi_l), offsetof(mps_2q_job, k),"
        " sizeof(mps_svd_params), sizeof(mps_1q_job), offsetof(mps_1q_job, chi_r));"
        " return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    size, off_status, off_chil, off_k, psize, size1, off_chir1 = map(int, out)
    assert size1 == _native.JOB1_DTYPE.itemsize
    assert off_chir1 == _native.JOB1_DTYPE.fields["chi_r"][1]
    dt = _native.JOB_DTYPE
    assert size == dt.itemsize
    assert off_status == dt.fields["status"][1]
    assert off_chil == dt.fields["chi_l"][1]
    assert off_k == dt.fields["k"][1]
    assert psize == ctypes.sizeof(_native.SvdParams)


def test_shape_plan_and_cost_shards():
    from mpsim_gb300 import circuits as C
    circ = C.workload("brickwork_64q_d40_chi256")
    one, two = C.gate_shapes(circ)
    assert sum(two.values()) == circ.n_two_qudit_gates == 1260
    assert sum(one.values()) == 64 * 40
    assert max(two) == (256, 256, 256)
    batch = C.qutrit_batch(8)
    shards = C.shard_by_cost(batch, 3)
    assert sorted(i for s in shards for i in s) == list(range(8))
    assert C.shard_by_cost(batch, 1) == [list(range(8))]
    assert [len(s) for s in C.shard_by_cost(batch[:2], 4)].count(0) == 2


def test_status_words_checked_after_the_call():
    """MPS._check_status: a finished call whose status words report a NaN/Inf
    raises MPS_ERR_NONFINITE; an unfinished one is kept for later unless the
    check blocks; clean ones recycle their host buffer."""
    import types
    import torch
    from mpsim_gb300 import _native
    from mpsim_gb300.core import MPS

    class Ev:
        def __init__(self, done):
            self.done = done

        def query(self):
            return self.done

        def synchronize(self):
            self.done = True

    me = types.SimpleNamespace(_status_pending=[], _status_free=[])
    clean = torch.zeros(4, dtype=torch.int32)
    bad = torch.tensor([0, _native.STATUS_NONFINITE, 0, 0], dtype=torch.int32)
    me._status_pending = [(clean, Ev(True)), (bad, Ev(False))]
    MPS._check_status(me, block=False)              # the unfinished one waits
    assert len(me._status_pending) == 1 and me._status_free == [clean]
    with pytest.raises(_native.NativeError) as ei:
        MPS._check_status(me, block=True)
    assert ei.value.code == _native.MPS_ERR_NONFINITE
    assert me._status_pending == []


def test_wide_split_compression_keeps_u_and_s(monkeypatch):
    """_wide_left_svd's column-block compression (the host logic of
    from_wavefunction's long splits), with the device SVD and GEMM replaced by
    NumPy: every level keeps mat mat^H, so U and S are those of mat, and the
    remainder U^H mat rebuilds it.  Covers several levels, a ragged last
    block and a matrix within the kernel's length."""
    import torch
    from mpsim_gb300 import core

    def fake_batch(device, stream, mats, left_canonical, on_unconverged="raise"):
        a = mats.numpy().astype(np.complex128)
        u, s, vh = np.linalg.svd(a, full_matrices=False)
        left = u if left_canonical else u * s[:, None, :]
        right = s[:, :, None] * vh if left_canonical else vh
        t = lambda x: torch.from_numpy(x.astype(np.complex64))
        return t(left), t(right), torch.from_numpy(s.astype(np.float32))

    def fake_cgemm(lib, stream, m, n, k, a, a_off, sam, sak, conj_a, b, b_off, sbk, sbn, conj_b,
                   c, c_off, scm, scn, batch=1, bsa=0, bsb=0, bsc=0):
        fa, fb = a.reshape(-1).numpy(), b.reshape(-1).numpy()
        A = fa[a_off + np.arange(m)[:, None] * sam + np.arange(k)[None, :] * sak]
        B = fb[b_off + np.arange(k)[:, None] * sbk + np.arange(n)[None, :] * sbn]
        C = (np.conj(A) if conj_a else A) @ (np.conj(B) if conj_b else B)
        c.reshape(-1)[c_off + (np.arange(m)[:, None] * scm + np.arange(n)[None, :] * scn).ravel()] = \
            torch.from_numpy(C.astype(np.complex64).ravel())

    monkeypatch.setattr(core, "_given_svd_batch", fake_batch)
    monkeypatch.setattr(core, "_cgemm", fake_cgemm)
    monkeypatch.setattr(core._native, "load", lambda: None)
    rng = np.random.default_rng(3)
    for m, n in ((2, 9000), (40, 5000), (700, 2100), (1200, 4000), (64, 1500)):
        mat = (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))).astype(np.complex64)
        u, rest = core._wide_left_svd("cpu", None, torch.from_numpy(mat))
        u, rest = u.numpy().astype(np.complex128), rest.numpy().astype(np.complex128)
        assert u.shape == (m, m) and rest.shape == (m, n)
        assert np.allclose(u.conj().T @ u, np.eye(m), atol=1e-4)
        assert np.allclose(u @ rest, mat, atol=1e-3 * np.abs(mat).max())
        s_ref = np.linalg.svd(mat.astype(np.complex128), compute_uv=False)
        s_got = np.sort(np.linalg.norm(rest, axis=1))[::-1]
        assert np.allclose(s_got, s_ref, rtol=1e-4)
    with pytest.raises(NotImplementedError):
        core._wide_left_svd("cpu", None, torch.zeros((core.MAX_SVD_LENGTH, 4000), dtype=torch.complex64))


def test_apply_interleaves_disjoint_swap_chains_exactly():
    """MPS.apply's scheduling, on a recording stand-in for the state: the
    adjacent steps it issues (SWAP chains of non-adjacent gates interleaved
    across disjoint site ranges, one-qudit gates and overlapping ranges ending
    a group) applied to a dense state vector give the in-order result, and the
    chains of disjoint gates do interleave."""
    from mpsim_gb300.gates import gate_tensor

    n = 7
    rng = np.random.default_rng(11)

    class Rec:
        track_norms = False

        def __init__(self):
            self.steps = []

        def _check_two_qudit(self, gate, i, j):
            assert 0 <= i < n and 0 <= j < n and i != j

        def _two_qudit_steps(self, gate, i, j, kw):
            return MPS._two_qudit_steps(self, gate, i, j, kw)

        def swap(self, a, b, **kw):
            self.steps.append(("2", np.asarray(gate_tensor(G.swap())), a, b))

        def apply_two_qudit_gate(self, gate, i, j, **kw):
            assert abs(i - j) == 1
            self.steps.append(("2", np.asarray(gate_tensor(gate)), i, j))

        def apply_one_qudit_gate(self, gate, i, **kw):
            self.steps.append(("1", np.asarray(gate_tensor(gate)), i))

    def dense(seq):
        psi = np.zeros((2,) * n, complex)
        psi[(0,) * n] = 1.0
        for st in seq:
            if st[0] == "1":
                psi = np.moveaxis(np.tensordot(st[1].reshape(2, 2), psi, axes=([1], [st[2]])), 0, st[2])
            else:
                g, i, j = st[1].reshape(2, 2, 2, 2), st[2], st[3]
                psi = np.moveaxis(np.tensordot(g, psi, axes=([2, 3], [i, j])), [0, 1], [i, j])
        return psi.reshape(-1)

    ops, ref = [], []
    for layer in range(3):
        for q in range(n):
            u = G.haar_random_matrix(1, 2, int(rng.integers(1 << 30)))
            ops.append(MPSOperation(G.Node(np.asarray(u)), q))
            ref.append(("1", np.asarray(u), q))
        for a, b in ((0, 3), (6, 4), (2, 5)):              # the last overlaps both
            u = np.asarray(G.haar_random_matrix(2, 2, int(rng.integers(1 << 30)))).reshape((2,) * 4)
            ops.append(MPSOperation(G.Node(u), (a, b)))
            ref.append(("2", u, a, b))
    rec = Rec()
    MPS.apply(rec, ops)
    assert np.allclose(dense(rec.steps), dense(ref), atol=1e-10)
    # the first steps of the (0, 3) and (6, 4) chains sit next to each other
    two = [s for s in rec.steps if s[0] == "2"]
    assert (two[0][2], two[0][3]) == (0, 1) and (two[1][2], two[1][3]) == (4, 5)
