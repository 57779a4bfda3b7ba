"""MPS state and operations with mpsim's API (mpsim/core.py), on one GPU.

Site tensors live on the GPU as torch complex64 tensors of shape
(chi_left, d, chi_right).  Every state-changing or state-reading operation
runs in the sm_103a kernels of ``libmpsim_gb300.so`` (see
include/mpsim_gb300.h); Python only validates arguments (with mpsim's
exception types and conditions), plans shapes and owns memory.  There is no
CPU fallback: without the library or a CUDA device the constructor raises.

Differences from the reference, all deliberate:
* complex64 storage throughout (the reference silently promotes to
  complex128 when it meets the float64 ``cnot``/``swap`` or complex128 Haar
  gates; here every gate is cast to complex64 first);
* the per-gate norm history ``_norms`` (mpsim/core.py:1160-1161, marked
  "TODO: Remove ... only for convenience in benchmarking") is opt-in via
  ``track_norms=True``: it is a full O(n d chi^3) sweep after every gate;
* two-qudit gates on adjacent pairs are deferred: ``apply_two_qudit_gate``
  (and ``apply``, the shorthands, the swap chains of non-adjacent gates)
  validates at once and queues the gate, and the queue runs as one batched
  launch when a gate shares a site with a queued one or anything reads the
  sites -- exact, because each merged matrix depends only on its own two
  sites; unitary one-qudit gates are queued too and launched together; a
  device error of a queued gate is raised by the call that runs the queue;
* ``get_node(s)`` return host copies (TensorNetwork-like nodes with the
  reference's initial axis order: physical axis first);
* ``from_wavefunction`` returns the reference's state in a mixed-canonical
  gauge (TensorNetwork's split_node puts sqrt(S) on both sides); its middle
  bond must stay below the Jacobi kernel's register-held column length of
  1792 (21 qubits, 13 qutrits), longer splits are compressed by column
  blocks first;
* ``sample`` draws from the same single-site marginals with the same NumPy
  global-RNG calls as the reference, computing all marginals in one device
  pass instead of one full contraction per site and sample.
"""

from __future__ import annotations

import ctypes
import math
import warnings
from copy import deepcopy
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _native, autotune
from .gates import (Node, cnot, gate_tensor, haar_random_unitary, hgate, is_hermitian,
                    is_unitary, rgate, swap, xgate)

try:
    import torch
except ImportError:  # pragma: no cover - torch is a hard dependency on GPU hosts
    torch = None


class CannotConvertToMPSOperation(Exception):
    pass


# ---------------------------------------------------------------------------
# Host-side helpers (pure Python; unit-tested on CPU)

def _edges_of(gate):
    """(number of dangling edges, number of connected edges, dims)."""
    t = gate_tensor(gate)
    dims = tuple(int(x) for x in t.shape)
    if hasattr(gate, "get_all_dangling") and hasattr(gate, "get_all_nondangling"):
        return len(gate.get_all_dangling()), len(gate.get_all_nondangling()), dims
    return len(dims), 0, dims


def kept_count(maxsvals: Optional[int], rank: int) -> int:
    """Singular values kept for ``max_singular_values=maxsvals``.

    TensorNetwork keeps ``s[:min(maxsvals, rank)]``; a negative value acts like
    a Python slice stop, which this reproduces.
    """
    if maxsvals is None:
        return rank
    return len(range(rank)[:min(int(maxsvals), rank)])


def parse_truncation(kwargs: dict, max_bond_dimension_of, index: int) -> Optional[int]:
    """``fraction`` / ``maxsvals`` handling of mpsim/core.py:1110-1130.

    ``index`` is min(node_index1, node_index2) after the swap network.
    Returns the ``max_singular_values`` argument (None keeps everything).
    """
    if "fraction" in kwargs and "maxsvals" in kwargs:
        raise ValueError("Only one of (fraction, maxsvals) can be provided as kwargs.")
    maxsvals = None
    if "fraction" in kwargs:
        fraction = kwargs.get("fraction")
        if not (0 <= fraction <= 1):
            raise ValueError("Keyword fraction must be between 0 and 1 but is", fraction)
        maxsvals = int(round(fraction * max_bond_dimension_of(index)))
    if "maxsvals" in kwargs:
        maxsvals = int(kwargs.get("maxsvals"))
    return maxsvals


def max_bond_dimensions(nqudits: int, d: int) -> List[int]:
    """mpsim/core.py:235-242."""
    half = [d ** (i + 1) for i in range(nqudits // 2)]
    out = half + list(reversed(half))
    if nqudits % 2 == 0:
        out.remove(d ** (nqudits // 2))
    return out


def _require_cuda():
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError(
            "mpsim_gb300 runs on a CUDA GPU only (no CPU fallback); no CUDA device is visible")
    return torch.device("cuda", torch.cuda.current_device())


class _Workspace:
    """Grow-only device scratch buffers, one pool per device."""

    def __init__(self):
        self._buf = {}

    def get(self, device, nbytes: int, slot: str = "main"):
        key = (str(device), slot)
        cur = self._buf.get(key)
        if cur is None or cur.numel() < nbytes:
            size = max(int(nbytes), 1 << 20)
            if cur is not None:
                size = max(size, int(cur.numel() * 1.25))
            cur = torch.empty(size, dtype=torch.uint8, device=device)
            self._buf[key] = cur
        return cur


_WS = _Workspace()


# Longest merged matrix the Jacobi kernel takes (rows held in registers).
MAX_SVD_LENGTH = 1792


def _cgemm(lib, stream, m, n, k, a, a_off, sam, sak, conj_a, b, b_off, sbk, sbn, conj_b,
           c, c_off, scm, scn, batch=1, bsa=0, bsb=0, bsc=0):
    """mps_cgemm on torch complex64 tensors; *_off are element offsets."""
    for z0 in range(0, max(batch, 1), 65535):
        nb = min(65535, max(batch, 1) - z0)
        _native.check(lib.mps_cgemm(
            stream, m, n, k,
            ctypes.c_void_p(a.data_ptr() + 8 * (a_off + z0 * bsa)), sam, sak, int(conj_a),
            ctypes.c_void_p(b.data_ptr() + 8 * (b_off + z0 * bsb)), sbk, sbn, int(conj_b),
            ctypes.c_void_p(c.data_ptr() + 8 * (c_off + z0 * bsc)), scm, scn, nb, bsa, bsb, bsc))


def _check_svd_rc(rc: int, on_unconverged: str = "raise") -> None:
    """Maps the two-qudit call's status to an exception.  A Jacobi SVD that hit
    its sweep cap (MPS_ERR_NOT_CONVERGED) raises like any device error unless
    the caller opted into ``on_unconverged="warn"``, which keeps the factors
    of the last sweep and issues a RuntimeWarning instead."""
    if rc == _native.MPS_OK:
        return
    if rc == _native.MPS_ERR_NOT_CONVERGED and on_unconverged == "warn":
        warnings.warn("mpsim_gb300: " + _native.last_error(), RuntimeWarning)
        return
    raise _native.NativeError(rc, _native.last_error())


def _given_svd_batch(device, stream, mats, left_canonical: bool, on_unconverged: str = "raise"):
    """Thin SVDs of nb device matrices of one shape (``mats``: nb x m x n
    complex64, each row-major) in one call of the two-qudit kernel's
    given-matrix jobs (MPS_JOB_THETA_GIVEN, d = 1), keeping all r = min(m, n)
    values.  Returns (left (nb, m, r), right (nb, r, n), singular values
    (nb, r) float32 on the device): left = U, right = S V^H when
    left_canonical, else left = U S, right = V^H."""
    lib = _native.load()
    nb, m, n = (int(x) for x in mats.shape)
    if max(m, n) > MAX_SVD_LENGTH:
        raise NotImplementedError(
            f"a {m} x {n} matrix is longer than the {MAX_SVD_LENGTH} rows the Jacobi SVD kernel "
            f"holds")
    r = min(m, n)
    mats = mats.contiguous()
    a_out = torch.empty((nb, m, r), dtype=torch.complex64, device=device)
    b_out = torch.empty((nb, r, n), dtype=torch.complex64, device=device)
    sv = torch.zeros((nb, max(r, 1)), dtype=torch.float32, device=device)
    status = torch.zeros(nb, dtype=torch.int32, device=device)
    table = np.zeros(nb, dtype=_native.JOB_DTYPE)
    for b in range(nb):
        row = table[b]
        row["a"], row["b"], row["gate"] = mats[b].data_ptr(), 0, 0
        row["flags"] = _native.JOB_THETA_GIVEN
        row["a_out"] = a_out[b].data_ptr() if a_out.numel() else 0
        row["b_out"] = b_out[b].data_ptr() if b_out.numel() else 0
        row["svals"], row["status"] = sv[b].data_ptr(), status[b].data_ptr()
        row["chi_l"], row["chi_m"], row["chi_r"], row["k"] = m, n, n, r
        row["keep_left_canonical"] = 1 if left_canonical else 0
    jobs = torch.from_numpy(table.view(np.uint8)).to(device)
    nbytes = lib.mps_2q_workspace_bytes(nb, m, n, 1)
    ws = _WS.get(device, nbytes, "2q")
    rc = lib.mps_apply_2q_batch(stream, ctypes.c_void_p(jobs.data_ptr()), nb, m, n, 1,
                                ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                                ctypes.byref(_native.SvdParams()))
    _check_svd_rc(rc, on_unconverged)
    return a_out, b_out, sv[:, :r]


def _given_svd(device, stream, mat, left_canonical: bool, on_unconverged: str = "raise"):
    """Thin SVD of a device matrix ``mat`` (m x n complex64, row-major); see
    _given_svd_batch.  Returns (left (m, r), right (r, n), singular values
    (r,) float32 on the host)."""
    m, n = (int(x) for x in mat.shape)
    left, right, sv = _given_svd_batch(device, stream, mat.reshape(1, m, n), left_canonical,
                                       on_unconverged)
    return left[0], right[0], sv[0].cpu().numpy()


def _wide_left_svd(device, stream, mat):
    """Left factor and remainder of a wide or square device matrix ``mat``
    (m x n complex64, row-major, m <= n): U (m x m, orthonormal columns) and
    U^H mat = S V^H (m x n), every value kept -- what one cut of
    from_wavefunction needs.  Matrices within the Jacobi kernel's length go
    to it directly.  A longer one (n > MAX_SVD_LENGTH, m < MAX_SVD_LENGTH) is
    first compressed by columns: mat = [B_1 .. B_t] with blocks of
    MAX_SVD_LENGTH columns (the last one shorter), each replaced by its U_i S_i
    (m x min(m, width)), which leaves mat mat^H = sum B_i B_i^H -- and so U
    and S -- unchanged; the blocks of one width go through one batched call,
    and the compression repeats until the matrix fits.  U is then the left
    factor of the compressed matrix and the remainder one GEMM against mat."""
    m, n = (int(x) for x in mat.shape)
    if n <= MAX_SVD_LENGTH:
        left, right, _ = _given_svd(device, stream, mat, True)
        return left, right
    if m >= MAX_SVD_LENGTH:
        raise NotImplementedError(
            f"a {m} x {n} matrix has both sides at or above the {MAX_SVD_LENGTH} rows the "
            f"Jacobi SVD kernel holds")
    ell = MAX_SVD_LENGTH
    c = mat.contiguous()
    while int(c.shape[1]) > ell:
        w = int(c.shape[1])
        full, tail = divmod(w, ell)
        parts = []
        if full:
            blocks = c[:, :full * ell].reshape(m, full, ell).permute(1, 0, 2)
            us, _, _ = _given_svd_batch(device, stream, blocks, False)
            parts.append(us.permute(1, 0, 2).reshape(m, full * m))
        if tail:
            us, _, _ = _given_svd(device, stream, c[:, full * ell:].contiguous(), False)
            parts.append(us)
        c = torch.cat(parts, dim=1).contiguous() if len(parts) > 1 else parts[0].contiguous()
    u, _, _ = _given_svd(device, stream, c, True)
    u = u.contiguous()
    rest = torch.empty((m, n), dtype=torch.complex64, device=device)
    _cgemm(_native.load(), stream, m, n, m, u, 0, 1, m, True, mat, 0, n, 1, False,
           rest, 0, n, 1)
    return u, rest


def kept_by_truncation_error(svals: np.ndarray, max_truncation_err: float) -> int:
    """Values TensorNetwork 0.2.1's split_node_full_svd keeps under
    max_truncation_err (what mpsim/core.py:876-881, 926-931 ask for): count of
    sqrt(cumsum(s[::-1]^2)) above the bound, i.e. the largest values whose
    dropped tail has norm <= the bound (computed in the values' dtype)."""
    s = np.asarray(svals)
    errs = np.sqrt(np.cumsum(np.square(s[::-1])))
    return int(np.count_nonzero(errs > max_truncation_err))


def _ptr_array(tensors):
    arr = (ctypes.c_void_p * len(tensors))()
    for i, t in enumerate(tensors):
        arr[i] = t.data_ptr() if t.numel() > 0 else 0
    return arr


def _int_array(vals):
    arr = (ctypes.c_int * len(vals))()
    for i, v in enumerate(vals):
        arr[i] = int(v)
    return arr


# ---------------------------------------------------------------------------

class MPSOperation:
    """An operation on one or two qudits (mpsim/core.py:21-156)."""

    def __init__(self, node, qudit_indices: Union[int, Tuple[int, ...]],
                 qudit_dimension: int = 2) -> None:
        self._node = node
        if isinstance(qudit_indices, (int, np.integer)):
            qudit_indices = (int(qudit_indices),)
        self._qudit_indices = tuple(qudit_indices)
        self._qudit_dimension = int(qudit_dimension)

    @property
    def qudit_indices(self) -> Tuple[int, ...]:
        return self._qudit_indices

    @property
    def qudit_dimension(self) -> int:
        return self._qudit_dimension

    @property
    def num_qudits(self) -> int:
        return len(self._qudit_indices)

    def node(self, copy: bool = True):
        if not copy:
            return self._node
        return Node(deepcopy(gate_tensor(self._node)), name=getattr(self._node, "name", None))

    def tensor(self, reshape_to_square_matrix: bool = True) -> np.ndarray:
        t = deepcopy(gate_tensor(self._node))
        if reshape_to_square_matrix:
            dim = self._qudit_dimension ** self.num_qudits
            t = np.reshape(t, (dim, dim))
        return t

    def is_valid(self) -> bool:
        d = self._qudit_dimension
        ndang, nconn, dims = _edges_of(self._node)
        if dims != tuple([d] * 2 * self.num_qudits):
            return False
        if ndang + nconn != 2 * self.num_qudits:
            return False
        if nconn:
            return False
        return True

    def is_unitary(self) -> bool:
        return is_unitary(self.tensor(reshape_to_square_matrix=True))

    def is_hermitian(self) -> bool:
        return is_hermitian(self.tensor(reshape_to_square_matrix=True))

    def is_single_qudit_operation(self) -> bool:
        return self.num_qudits == 1

    def is_two_qudit_operation(self) -> bool:
        return self.num_qudits == 2

    def __str__(self):
        return f"Tensor {getattr(self._node, 'name', '')} on qudit(s) {self._qudit_indices}."


class MPS:
    """Matrix product state on one GPU (mpsim/core.py:159-1423)."""

    def __init__(self, nqudits: int, qudit_dimension: int = 2, tensor_prefix: str = "q",
                 *, track_norms: bool = False, record_svals: bool = False,
                 on_unconverged: str = "raise", precision: str = "plain",
                 autotune: bool = True) -> None:
        if nqudits < 2:
            raise ValueError(f"Number of qudits must be greater than 2 but is {nqudits}.")
        self._nqudits = int(nqudits)
        self._qudit_dimension = int(qudit_dimension)
        self._prefix = tensor_prefix
        self._max_bond_dimensions = max_bond_dimensions(self._nqudits, self._qudit_dimension)
        self._norms = []  # type: List[float]
        self.track_norms = track_norms
        self.record_svals = record_svals
        self.svals_history = []
        self.svd_params = _native.SvdParams()
        if on_unconverged not in ("raise", "warn"):
            raise ValueError("on_unconverged must be 'raise' or 'warn'")
        # a Jacobi SVD that hits its sweep cap raises NativeError (or, with
        # "warn", keeps the last sweep's factors and warns)
        self.on_unconverged = on_unconverged
        if precision not in ("plain", "mixed", "auto"):
            raise ValueError("precision must be 'plain', 'mixed' or 'auto'")
        # "plain": complex64 on FP32 SIMT throughout.  "mixed": the truncated
        # SVDs of left-canonical tall gates of 64+ columns run as tensor-core
        # block sweeps (split-bf16 tcgen05 Gram and rotation GEMMs, FP64
        # off-diagonal test); every other gate runs the plain form.  "auto":
        # for those gates, whichever of the two the autotuner's table found
        # faster for the call's shape and batch.
        self.precision = precision
        # per-call solver settings (LQ preconditioning, block width) from the
        # autotuner's table (mpsim_gb300.autotune); False keeps the defaults
        self.autotune = autotune
        # When a list, each batched two-qudit launch appends
        # (jobs, max_m, max_n, sweeps, start_event, end_event).
        self.timing = None
        self._device = _require_cuda()
        # Two-qudit gates on adjacent pairs wait here until a gate that shares
        # a site, or any operation that reads or rewrites sites, needs them;
        # then they run as one batched launch (see _sites).
        self._pending = []
        self._pending_sites = set()
        self._pending_1q = []            # (site, d x d complex64 gate) waiting for one launch
        self._pending_1q_sites = set()
        # per-job status words of earlier two-qudit calls, copied to pinned
        # host memory behind each call and checked once the copy is done
        self._status_pending = []
        self._status_free = []           # pinned buffers of checked calls, reused
        # bumped whenever a site tensor is replaced; is_valid caches per value
        self._version = 0
        self._valid_at = (-1, False)
        d = self._qudit_dimension
        init = torch.zeros((self._nqudits, 1, d, 1), dtype=torch.complex64)
        init[:, 0, 0, 0] = 1.0
        init = init.to(self._device)
        self._site_list = [init[i].clone() for i in range(self._nqudits)]

    @classmethod
    def from_sites(cls, sites, qudit_dimension: int, **kwargs) -> "MPS":
        """An MPS around existing device site tensors ((chi_l, d, chi_r)
        complex64, shared, not copied), e.g. a CircuitPlan's final state."""
        sites = list(sites)
        mps = cls(len(sites), qudit_dimension, **kwargs)
        for t in sites:
            if t.dtype != torch.complex64 or t.dim() != 3 or int(t.shape[1]) != mps._qudit_dimension:
                raise ValueError("sites must be (chi_l, d, chi_r) complex64 tensors")
        mps._site_list = sites
        mps._version += 1
        return mps

    # -- deferred two-qudit gates ---------------------------------------------
    # apply_two_qudit_gate validates at once (the reference's exceptions) and
    # queues the gate; gates on disjoint adjacent pairs commute, so applying
    # the queue as one batch gives exactly the result of applying them one by
    # one, and gate-by-gate callers get the batched kernels.  Every access to
    # _sites runs the queue first; only the queueing path itself (validity,
    # kept-count planning for a pair no queued gate touches, one-qudit gates
    # on such sites) and the flush read _site_list directly.  A device error of
    # a queued gate (NaN, timeout) is raised by the call that flushes it.
    # Unitary one-qudit gates are queued the same way and launched together
    # (one copy of all their matrices, one mps_apply_1q_batch): they touch no
    # site a queued two-qudit gate touches, and at most one gate per site is
    # queued, so the order of launch among them is free.
    @property
    def _sites(self):
        if self._pending or self._pending_1q:
            self._flush()
        return self._site_list

    @_sites.setter
    def _sites(self, value):
        if self._pending or self._pending_1q:
            self._flush()
        self._site_list = value
        self._version += 1

    def _flush(self) -> None:
        """Runs the queued one-qudit gates, then the queued two-qudit gates
        (disjoint sites), each queue as one batched launch."""
        self._flush_1q()
        pending = self._pending
        self._pending = []
        self._pending_sites = set()
        if pending:
            self._run_pairs(pending)

    def _flush_1q(self) -> None:
        pending = self._pending_1q
        if not pending:
            return
        self._pending_1q = []
        self._pending_1q_sites = set()
        d, n1 = self._qudit_dimension, len(pending)
        mats = np.ascontiguousarray(np.stack([m for _, m in pending]).astype(np.complex64))
        g = torch.from_numpy(mats).to(self._device)
        table = np.zeros(n1, dtype=_native.JOB1_DTYPE)
        for q, (i, _) in enumerate(pending):
            site = self._site_list[i]
            table[q]["site"] = site.data_ptr()
            table[q]["gate"] = g[q].data_ptr()
            table[q]["chi_l"], table[q]["chi_r"] = int(site.shape[0]), int(site.shape[2])
        jt = torch.from_numpy(table.view(np.uint8)).to(self._device)
        _native.check(self._lib().mps_apply_1q_batch(self._stream(), ctypes.c_void_p(jt.data_ptr()),
                                                     n1, d))

    def _touches_pending(self, *sites) -> bool:
        return any(s in self._pending_sites for s in sites)

    def _touches_pending_1q(self, *sites) -> bool:
        return any(s in self._pending_1q_sites for s in sites)

    # -- plumbing ----------------------------------------------------------
    @property
    def device(self):
        return self._device

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self._device).cuda_stream)

    def _lib(self):
        return _native.load()

    def _to_device_gate(self, mat: np.ndarray):
        g = np.ascontiguousarray(np.asarray(mat).astype(np.complex64))
        return torch.from_numpy(g).to(self._device)

    @property
    def sites(self):
        """The device site tensors, (chi_left, d, chi_right) complex64."""
        return list(self._sites)

    # -- structure ---------------------------------------------------------
    @property
    def nqudits(self) -> int:
        return self._nqudits

    @property
    def qudit_dimension(self) -> int:
        return self._qudit_dimension

    def bond_dimension_of(self, node_index: int) -> int:
        if not self.is_valid():
            raise ValueError("MPS is invalid.")
        if node_index >= self._nqudits:
            raise ValueError(f"Index should be less than {self._nqudits} but is {node_index}.")
        if node_index == self._nqudits - 1:
            raise IndexError("list index out of range")
        if node_index < 0:
            if self._nqudits == 2 and node_index == -1:
                raise ValueError("Non-connected graph")
            raise ValueError("Non-connected graph")
        return int(self._sites[node_index].shape[2])

    def bond_dimensions(self) -> List[int]:
        return [self.bond_dimension_of(i) for i in range(self._nqudits - 1)]

    def max_bond_dimension_of(self, edge_index: int) -> int:
        if edge_index >= self._nqudits:
            raise ValueError(f"Edge index should be less than {self._nqudits} but is {edge_index}.")
        return self._max_bond_dimensions[edge_index]

    def max_bond_dimensions(self) -> List[int]:
        return self._max_bond_dimensions

    def is_valid(self) -> bool:
        # queued gates keep every bond consistent, so the current list answers;
        # the answer only changes when a site tensor is replaced (_version)
        if self._valid_at[0] == self._version:
            return self._valid_at[1]
        ok = self._check_valid()
        self._valid_at = (self._version, ok)
        return ok

    def _check_valid(self) -> bool:
        s = self._site_list
        if len(s) < 2:
            return False
        d = self._qudit_dimension
        if s[0].shape[0] != 1 or s[-1].shape[2] != 1:
            return False
        for i, t in enumerate(s):
            if t.dim() != 3 or t.shape[1] != d:
                return False
            if i < len(s) - 1 and t.shape[2] != s[i + 1].shape[0]:
                print(f"Nodes at index {i} and {i + 1} are not connected.")
                return False
        return True

    def _chis(self, sites=None):
        sites = self._sites if sites is None else sites
        return [int(sites[0].shape[0])] + [int(t.shape[2]) for t in sites]

    def get_nodes(self, copy: bool = True) -> List[Node]:
        """Host copies of the site tensors, physical axis first:
        (d, chi) for the end sites, (d, chi_left, chi_right) inside."""
        out = []
        n = self._nqudits
        for i, t in enumerate(self._sites):
            a = t.detach().cpu().numpy()
            a = np.transpose(a, (1, 0, 2))
            if i == 0:
                a = a[:, 0, :]
            elif i == n - 1:
                a = a[:, :, 0]
            out.append(Node(a.copy(), name=self._prefix + str(i)))
        return out

    def get_node(self, node_index: int, copy: bool = True) -> Node:
        return self.get_nodes(copy)[node_index]

    # -- contractions ------------------------------------------------------
    def wavefunction(self) -> np.ndarray:
        """Full state vector, qudit 0 most significant (core.py:483-500)."""
        if not self.is_valid():
            raise ValueError("MPS is not valid.")
        d, n = self._qudit_dimension, self._nqudits
        size = d ** n
        if size > (1 << 31):
            raise ValueError(f"wavefunction of {size} amplitudes is too large")
        chis = self._chis()
        need, p = 1, 1
        for i in range(n):
            p *= d
            need = max(need, p * max(chis[i + 1], 1))
        ws = _WS.get(self._device, 2 * need * 8, "wf")
        out = torch.empty(size, dtype=torch.complex64, device=self._device)
        _native.check(self._lib().mps_wavefunction(
            self._stream(), _ptr_array(self._sites), _int_array(chis), n, d,
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ws.numel()))
        res = out.cpu().numpy()
        self._check_status(block=True)
        return res

    def amplitudes(self, bitstrings) -> np.ndarray:
        """<x|psi> for each row of ``bitstrings`` (shape (S, nqudits))."""
        bits = np.ascontiguousarray(np.asarray(bitstrings, dtype=np.int8))
        if bits.ndim != 2 or bits.shape[1] != self._nqudits:
            raise ValueError("bitstrings must have shape (count, nqudits)")
        if bits.size and (bits.min() < 0 or bits.max() >= self._qudit_dimension):
            raise ValueError("bitstring digits must lie in [0, qudit_dimension)")
        nb = bits.shape[0]
        if nb == 0:
            return np.zeros(0, np.complex64)
        chis = self._chis()
        mx = max(chis)
        d = self._qudit_dimension
        ws = _WS.get(self._device, (nb * d * mx + 2 * nb * mx) * 8, "amp")
        bdev = torch.from_numpy(bits).to(self._device)
        out = torch.empty(nb, dtype=torch.complex64, device=self._device)
        _native.check(self._lib().mps_amplitudes(
            self._stream(), _ptr_array(self._sites), _int_array(chis), self._nqudits, d,
            ctypes.c_void_p(bdev.data_ptr()), nb, ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(ws.data_ptr()), ws.numel()))
        res = out.cpu().numpy()
        self._check_status(block=True)
        return res

    def dagger(self) -> None:
        """Conjugates every site (core.py:502-505)."""
        for t in self._sites:
            _native.check(self._lib().mps_scale(self._stream(), ctypes.c_void_p(t.data_ptr()),
                                                t.numel(), 1.0, 0.0, 1))

    def inner_product(self, other: "MPS") -> complex:
        """sum_x self(x) * conj(other(x)) (core.py:507-561)."""
        if other._nqudits != self._nqudits:
            raise ValueError(
                f"Cannot compute inner product between self which has {self._nqudits} qudits "
                f"and other which has {other._nqudits} qudits.\nNumber of qudits must be equal.")
        if other._qudit_dimension != self._qudit_dimension:
            raise ValueError(
                f"Cannot compute inner product between self which has qudit dimension "
                f"{self._qudit_dimension} and other which as qudit dimension "
                f"{other._qudit_dimension}.Qudit dimensions must be equal.")
        if not self.is_valid():
            raise ValueError("MPS is invalid.")
        if not other.is_valid():
            raise ValueError("Other MPS is invalid.")
        ca, cb = self._chis(), other._chis()
        mx = max(max(ca), max(cb))
        nbytes = self._lib().mps_sweep_workspace_bytes(mx, self._qudit_dimension)
        ws = _WS.get(self._device, nbytes, "sweep")
        res = (ctypes.c_double * 2)()
        _native.check(self._lib().mps_inner_product(
            self._stream(), _ptr_array(self._sites), _int_array(ca), _ptr_array(other._sites),
            _int_array(cb), self._nqudits, self._qudit_dimension, ctypes.c_void_p(ws.data_ptr()),
            ws.numel(), res))
        return complex(res[0], res[1])

    def norm(self) -> float:
        """sqrt(Re <self|self>) (core.py:563-565)."""
        n = np.sqrt(self.inner_product(self).real)
        self._check_status(block=True)
        return n

    def _check_status(self, block: bool) -> None:
        """Raises NativeError(MPS_ERR_NONFINITE) for a finished two-qudit call
        whose per-job status words report a NaN/Inf singular value that first
        appeared after the call returned (one in theta, a sweep cap or an
        expired wait the call reports itself).  block=False looks only at the
        calls whose status copy has completed."""
        keep = []
        for st_host, ev in self._status_pending:
            if not block and not ev.query():
                keep.append((st_host, ev))
                continue
            ev.synchronize()
            bits = int(np.bitwise_or.reduce(st_host.numpy())) if st_host.numel() else 0
            if bits & _native.STATUS_NONFINITE:
                self._status_pending = []
                raise _native.NativeError(_native.MPS_ERR_NONFINITE,
                                          "a two-qudit gate produced a NaN/Inf singular value")
            self._status_free.append(st_host)
        self._status_pending = keep

    def renormalize(self, to_norm: float = 1.0) -> None:
        """Scales every site by (to_norm / norm)^(1/n) (core.py:567-594)."""
        if to_norm < 0.0:
            raise ValueError(f"Arg to_norm must be positive but is {to_norm}")
        if np.isclose(to_norm, 0.0, atol=1e-15):
            raise ValueError(f"Arg to_norm = {to_norm} is too close to numerical zero.")
        norm = self.norm()
        if np.isclose(norm, 0.0, atol=1e-15):
            raise ValueError("Norm of MPS is numerically zero, cannot renormalize.")
        factor = float((to_norm / norm) ** (1 / self._nqudits))
        for t in self._sites:
            _native.check(self._lib().mps_scale(self._stream(), ctypes.c_void_p(t.data_ptr()),
                                                t.numel(), factor, 0.0, 0))

    def expectation(self, observable: MPSOperation) -> float:
        """<mps|O|mps> (core.py:723-751)."""
        if not observable.is_hermitian():
            raise ValueError("Observable is not Hermitian.")
        if observable.qudit_dimension != self._qudit_dimension:
            od, md = observable.qudit_dimension, self._qudit_dimension
            raise ValueError(
                f"Dimension mismatch between observable and MPS. Observable is ({od}, {od}) "
                f"but MPS has qudit dimension {md}.")
        other = self.copy()
        other.apply(observable)
        return self.inner_product(other).real

    def reduced_density_matrix(self, node_indices) -> np.ndarray:
        """rho[(ket digits), (bra digits)] on ``node_indices`` (in that order),
        every other site traced out (core.py:596-653); not normalised.  One
        left-to-right environment sweep on the device: E[b, l, l'] with b the
        digits of the sites kept so far, two batched complex GEMMs per site."""
        try:
            node_indices = iter(node_indices)
        except TypeError:
            node_indices = [node_indices]
        node_indices = tuple(node_indices)
        if len(set(node_indices)) < len(node_indices):
            raise ValueError("Node indices contains duplicates.")
        if min(node_indices) < 0 or max(node_indices) > self._nqudits - 1:
            raise IndexError("One or more invalid node indices.")
        d, dev = self._qudit_dimension, self._device
        lib, stream = self._lib(), self._stream()
        kept = sorted(node_indices)
        keep_set = set(kept)
        E = torch.ones((1, 1, 1), dtype=torch.complex64, device=dev)
        nb = 1
        for i, A in enumerate(self._sites):
            cl, _, cr = (int(x) for x in A.shape)
            # F[b, l', (a, r)] = sum_l E[b, l, l'] A[l, (a, r)]
            F = torch.empty((nb, cl, d, cr), dtype=torch.complex64, device=dev)
            _cgemm(lib, stream, cl, d * cr, cl, E, 0, 1, cl, 0, A, 0, d * cr, 1, 0,
                   F, 0, d * cr, 1, nb, cl * cl, 0, cl * d * cr)
            if i in keep_set:
                # E'[b, a, a', r, r'] = sum_l' F[b, l', a, r] conj(A[l', a', r'])
                E = torch.empty((nb, d, d, cr, cr), dtype=torch.complex64, device=dev)
                for a in range(d):
                    for a2 in range(d):
                        _cgemm(lib, stream, cr, cr, cl, F, a * cr, 1, d * cr, 0,
                               A, a2 * cr, d * cr, 1, 1, E, (a * d + a2) * cr * cr, cr, 1,
                               nb, cl * d * cr, 0, d * d * cr * cr)
                nb *= d * d
                E = E.view(nb, cr, cr)
            else:
                # E'[b, r, r'] = sum_(l', a) F[b, (l', a), r] conj(A[(l', a), r'])
                E = torch.empty((nb, cr, cr), dtype=torch.complex64, device=dev)
                _cgemm(lib, stream, cr, cr, cl * d, F, 0, 1, cr, 0, A, 0, cr, 1, 1,
                       E, 0, cr, 1, nb, cl * d * cr, 0, cr * cr)
        k = len(kept)
        vals = E.reshape(nb).cpu().numpy().reshape((d,) * (2 * k))
        pos = {site: p for p, site in enumerate(kept)}
        perm = [2 * pos[i] for i in node_indices] + [2 * pos[i] + 1 for i in node_indices]
        return np.ascontiguousarray(vals.transpose(perm)).reshape(d ** k, d ** k)

    def site_marginals(self) -> np.ndarray:
        """(nqudits, d) float32: the diagonal of every single-site reduced
        density matrix (not normalised), from one device pass."""
        if not self.is_valid():
            raise ValueError("MPS is invalid.")
        d, n = self._qudit_dimension, self._nqudits
        chis = _int_array(self._chis())
        lib = self._lib()
        ws = _WS.get(self._device, lib.mps_marginals_workspace_bytes(chis, n, d), "marg")
        out = np.zeros((n, d), dtype=np.float32)
        _native.check(lib.mps_site_marginals(
            self._stream(), _ptr_array(self._sites), chis, n, d, ctypes.c_void_p(ws.data_ptr()),
            ws.numel(), out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def sample(self, nsamples: int, as_hist: bool = False, as_string: bool = False):
        """Samples as MPS.sample does (core.py:669-709): each site's digit is
        drawn with np.random.choice from that site's marginal,
        reduced_density_matrix(i).diagonal().real (core.py:655-667), in the
        same order of NumPy global-RNG calls, so a seeded np.random gives the
        reference's draws; the marginals come from one device pass."""
        if not isinstance(nsamples, int):
            raise ValueError(f"Arg nsamples should be an int but is a {type(nsamples)}.")
        if nsamples <= 0:
            raise ValueError(f"Arg nsamples should be positive but is {nsamples}.")
        if as_hist:
            as_string = True
        probs = self.site_marginals()
        states = list(range(self._qudit_dimension))
        raw = []
        for _ in range(nsamples):
            string = [np.random.choice(states, size=1, p=probs[i])[0]
                      for i in range(self._nqudits)]
            raw.append("".join(str(bit) for bit in string) if as_string else string)
        if as_hist:
            hist = {}
            for bitstring in raw:
                hist[bitstring] = hist.get(bitstring, 0) + 1
            return hist
        return raw

    @staticmethod
    def from_wavefunction(wavefunction, nqudits: int, qudit_dimension: int = 2,
                          tensor_prefix: str = "q") -> "MPS":
        """MPS of a state vector by successive SVDs across every cut, all
        singular values kept (core.py:245-328): the reference's state and bond
        dimensions min(d^i, d^(n-i)).  The gauge differs (TensorNetwork's
        split_node puts sqrt(S) on both sides): the cuts left of the middle
        site are split from the left (U on each site, S V^H carried right),
        the others from the right end on the conjugate transpose (V^H on each
        site, U S carried left), so that every split is of a wide matrix whose
        short side is the bond (_wide_left_svd).  The middle cut's bond must
        stay below the Jacobi kernel's 1792 rows: up to 21 qubits or 13
        qutrits."""
        if not isinstance(wavefunction, (list, tuple, np.ndarray)):
            raise TypeError("Invalid type for wavefunction.")
        wavefunction = np.array(wavefunction)
        if len(wavefunction.shape) != 1:
            raise ValueError("Invalid shape for wavefunction. Should be a vector.")
        if nqudits < 2:
            raise ValueError("At least two qudits are required.")
        d = int(qudit_dimension)
        if wavefunction.size != d ** nqudits:
            raise ValueError(
                "Mismatch between wavefunction, qudit_dimension, and nqudits. "
                f"Expected {d ** nqudits} elements in the wavefunction, but wavefunction has "
                f"{wavefunction.size} elements.")
        middle = nqudits // 2
        if d ** middle >= MAX_SVD_LENGTH:
            raise NotImplementedError(
                f"the middle bond of {nqudits} qudits of dimension {d} reaches the "
                f"{MAX_SVD_LENGTH} rows the Jacobi SVD kernel holds")
        mps = MPS(nqudits, d, tensor_prefix)
        dev, stream = mps._device, mps._stream()
        rest = torch.from_numpy(np.ascontiguousarray(wavefunction.astype(np.complex64))).to(dev)
        # sites 0 .. middle-1 from the left: rest (chi*d x d^(n-1-i)) = U . S V^H
        chi = 1
        sites = []
        for i in range(middle):
            u, rest = _wide_left_svd(dev, stream, rest.reshape(chi * d, d ** (nqudits - 1 - i)))
            k = int(u.shape[1])
            sites.append(u.reshape(chi, d, k))
            chi = k
        # sites n-1 .. middle+1 from the right: rest (rows x d*chir) = (U S) . V^H,
        # from the wide split of its conjugate transpose: rest^H = V . (S U^H)
        chir = 1
        right_sites = []
        rows = int(rest.numel()) // d
        for j in range(nqudits - 1, middle, -1):
            mat = rest.reshape(rows, d * chir)
            v, sut = _wide_left_svd(dev, stream, mat.conj().T.contiguous())
            k = int(v.shape[1])
            right_sites.append(v.conj().T.contiguous().reshape(k, d, chir))
            rest = sut.conj().T.contiguous()          # rows x k: U S
            chir = k
            rows //= d
        sites.append(rest.reshape(chi, d, chir))
        sites.extend(reversed(right_sites))
        mps._sites = sites
        return mps

    def orthonormalize_right_edge_of(self, node_index: int, threshold: float = 1e-8) -> None:
        """SVD of site i with rows (left bond, digit): site i <- U, site i+1
        <- S V^H . site i+1, dropping the smallest values whose tail norm is
        <= threshold * norm (core.py:847-891)."""
        if not 0 <= node_index < self._nqudits - 1:
            raise ValueError("Invalid edge index.")
        i = node_index
        node = self._sites[i]
        cl, d, cr = (int(x) for x in node.shape)
        max_err = threshold * self.norm()
        left, right, s = _given_svd(self._device, self._stream(), node.reshape(cl * d, cr), True,
                                     self.on_unconverged)
        keep = kept_by_truncation_error(s, max_err)
        r = int(left.shape[1])
        nxt = self._sites[i + 1]
        c2 = int(nxt.shape[2])
        new_next = torch.empty((keep, d, c2), dtype=torch.complex64, device=self._device)
        _cgemm(self._lib(), self._stream(), keep, d * c2, cr, right, 0, cr, 1, 0,
               nxt, 0, d * c2, 1, 0, new_next, 0, d * c2, 1)
        self._sites[i] = left[:, :keep].reshape(cl, d, keep) if keep == r else \
            left[:, :keep].contiguous().reshape(cl, d, keep)
        self._sites[i + 1] = new_next
        self._version += 1

    def orthonormalize_left_edge_of(self, node_index: int, threshold: float = 1e-8) -> None:
        """SVD of site i with columns (digit, right bond): site i <- V^H,
        site i-1 <- site i-1 . U S, dropping the smallest values whose tail
        norm is <= threshold * norm (core.py:893-937)."""
        if not 0 < node_index <= self._nqudits - 1:
            raise ValueError("Invalid edge index.")
        i = node_index
        node = self._sites[i]
        cl, d, cr = (int(x) for x in node.shape)
        max_err = threshold * self.norm()
        left, right, s = _given_svd(self._device, self._stream(), node.reshape(cl, d * cr), False,
                                     self.on_unconverged)
        keep = kept_by_truncation_error(s, max_err)
        r = int(left.shape[1])
        prev = self._sites[i - 1]
        c0 = int(prev.shape[0])
        new_prev = torch.empty((c0, d, keep), dtype=torch.complex64, device=self._device)
        _cgemm(self._lib(), self._stream(), c0 * d, keep, cl, prev, 0, cl, 1, 0,
               left, 0, r, 1, 0, new_prev, 0, keep, 1)
        self._sites[i] = right[:keep].reshape(keep, d, cr)
        self._sites[i - 1] = new_prev
        self._version += 1

    # -- one-qudit gates ---------------------------------------------------
    def _check_one_qudit(self, gate, node_index):
        if not self.is_valid():
            raise ValueError("MPS is invalid.")
        if node_index not in range(self._nqudits):
            raise ValueError(f"Input tensor index={node_index} is out of bounds for"
                             f" an MPS on {self._nqudits} qudits.")
        ndang, nconn, dims = _edges_of(gate)
        if ndang != 2 or nconn != 0:
            raise ValueError("Single qudit gate must have two free edges and zero connected edges.")
        if dims[0] != dims[1]:
            raise ValueError("Gate edge dimensions must be equal.")
        if dims[0] != self._qudit_dimension:
            raise ValueError(f"Gate edges have dimension {dims[0]} but should have MPS qudit "
                             f"dimension = {self._qudit_dimension}")

    def apply_one_qudit_gate(self, gate, node_index: int, **kwargs) -> None:
        """site[l,a',r] = sum_a U[a',a] site[l,a,r] (core.py:753-845)."""
        self._check_one_qudit(gate, node_index)
        mat = gate_tensor(gate)
        unitary = is_unitary(np.asarray(mat))
        if unitary:
            # queued (see _flush_1q); a queued gate on the same site runs first
            if self._touches_pending(node_index) or self._touches_pending_1q(node_index):
                self._flush()
            # a copy: the caller may reuse its array before the queue runs
            self._pending_1q.append((node_index, np.array(mat, dtype=np.complex64)))
            self._pending_1q_sites.add(node_index)
            return
        renorm = kwargs.get("renormalize_after_non_unitary") is not False
        ortho = kwargs.get("ortho_after_non_unitary") is not False
        norm = self.norm() if (not unitary and renorm) else None
        if self._touches_pending(node_index) or self._pending_1q:
            self._flush()
        site = self._site_list[node_index]
        g = self._to_device_gate(mat)
        _native.check(self._lib().mps_apply_1q(
            self._stream(), ctypes.c_void_p(site.data_ptr()), int(site.shape[0]),
            self._qudit_dimension, int(site.shape[2]), ctypes.c_void_p(g.data_ptr())))
        if not unitary and ortho:
            # core.py:828-842
            if node_index == 0:
                self.orthonormalize_right_edge_of(node_index)
            elif node_index == self._nqudits - 1:
                self.orthonormalize_left_edge_of(node_index)
            else:
                self.orthonormalize_right_edge_of(node_index)
                self.orthonormalize_left_edge_of(node_index)
        if norm is not None:
            self.renormalize(norm)

    def _apply_one_qudit_layer(self, one_qudit) -> None:
        """One-qudit gates on every site (``one_qudit``: (n, d, d)) in one
        batched launch; non-unitary gates take the per-gate path."""
        d, n = self._qudit_dimension, self._nqudits
        if isinstance(one_qudit, (list, tuple)):
            u = np.stack([np.asarray(gate_tensor(x)) for x in one_qudit])
        else:
            u = np.asarray(gate_tensor(one_qudit))
        if u.shape != (n, d, d):
            raise ValueError(f"one-qudit layer must have shape ({n}, {d}, {d})")
        prod = np.einsum("nji,njk->nik", u.conj(), u)
        if not np.allclose(prod, np.broadcast_to(np.identity(d), prod.shape), atol=1e-5):
            for i in range(n):
                self.apply_one_qudit_gate(u[i], i)
            return
        if not self.is_valid():
            raise ValueError("MPS is invalid.")
        g = torch.from_numpy(np.ascontiguousarray(u.astype(np.complex64))).to(self._device)
        table = np.zeros(n, dtype=_native.JOB1_DTYPE)
        for i, site in enumerate(self._sites):
            table[i]["site"] = site.data_ptr()
            table[i]["gate"] = g[i].data_ptr()
            table[i]["chi_l"], table[i]["chi_r"] = int(site.shape[0]), int(site.shape[2])
        jt = torch.from_numpy(table.view(np.uint8)).to(self._device)
        _native.check(self._lib().mps_apply_1q_batch(self._stream(), ctypes.c_void_p(jt.data_ptr()),
                                                     n, d))

    def apply_one_qudit_gate_to_all(self, gate) -> None:
        for i in range(self._nqudits):
            self.apply_one_qudit_gate(gate, i)

    # -- two-qudit gates ---------------------------------------------------
    def _check_two_qudit(self, gate, i, j):
        if not self.is_valid():
            raise ValueError("MPS is not valid.")
        if i not in range(self._nqudits) or j not in range(self._nqudits):
            raise ValueError(f"Input tensor indices={(i, j)} are out of "
                             f"bounds for an MPS on {self._nqudits} qudits.")
        if i == j:
            raise ValueError("Node indices cannot be identical.")
        ndang, nconn, dims = _edges_of(gate)
        if ndang != 4 or nconn != 0:
            raise ValueError("Two qubit gate must have four free edges and zero connected edges.")
        if len(set(dims)) != 1:
            raise ValueError("All gate edges must have the same dimension.")
        if dims[0] != self._qudit_dimension:
            raise ValueError(f"Gate edges have dimension {dims[0]} but should have MPS qudit "
                             f"dimension = {self._qudit_dimension}")

    def _prepare_pair(self, gate, i, j, kwargs, checked=False):
        """Validate, flip, and return (G (d^2 x d^2) complex64, left, k, lc)
        for an ADJACENT pair.  Mirrors core.py:1000-1033 and 1104-1130.
        ``checked``: the caller already verified that the MPS is valid."""
        if checked:
            if i not in range(self._nqudits) or j not in range(self._nqudits) or i == j:
                raise ValueError(f"Input tensor indices={(i, j)} are out of bounds for an MPS on "
                                 f"{self._nqudits} qudits.")
            dims = tuple(int(x) for x in np.shape(gate_tensor(gate)))
            if len(dims) != 4 or len(set(dims)) != 1 or dims[0] != self._qudit_dimension:
                raise ValueError("Two qudit gate must be (d, d, d, d) with the MPS qudit dimension.")
        else:
            self._check_two_qudit(gate, i, j)
        d = self._qudit_dimension
        g = np.asarray(gate_tensor(gate)).reshape((d,) * 4)
        if j < i:
            g = g.transpose(1, 0, 3, 2)
            i, j = j, i
        lc = kwargs["keep_left_canonical"] if "keep_left_canonical" in kwargs else True
        maxsvals = parse_truncation(kwargs, self.max_bond_dimension_of, min(i, j))
        if self._touches_pending(i, j):
            self._flush()
        elif self._touches_pending_1q(i, j):
            self._flush_1q()              # those one-qudit gates come first
        a, b = self._site_list[i], self._site_list[j]
        m = int(a.shape[0]) * d
        n = int(b.shape[2]) * d
        k = kept_count(maxsvals, min(m, n))
        return g.reshape(d * d, d * d).astype(np.complex64), i, k, bool(lc)

    def apply_two_qudit_gate(self, gate, node_index1: int, node_index2: int, **kwargs) -> None:
        """Two-qudit gate with truncated SVD (core.py:950-1161)."""
        self._check_two_qudit(gate, node_index1, node_index2)
        d = self._qudit_dimension
        g = np.asarray(gate_tensor(gate)).reshape((d,) * 4)
        i, j = node_index1, node_index2
        if j < i:
            g = g.transpose(1, 0, 3, 2)
            i, j = j, i
        invert = False
        if i < j - 1:
            invert = True
            original = i
            self.move_node_from_left_to_right(i, j - 1, **kwargs)
            i = j - 1
        pair = self._prepare_pair(g, i, j, kwargs)      # flushes a queued gate on i or j
        self._pending.append(pair)
        self._pending_sites.update((pair[1], pair[1] + 1))
        if invert:
            self.move_node_from_right_to_left(i, original, **kwargs)
        if self.track_norms:
            self._norms.append(self.norm())

    def _run_pairs(self, pairs):
        """One batched launch for two-qudit gates on disjoint adjacent pairs.
        With precision="mixed" the call is MPS_PRECISION_MIXED: the gates the
        tensor-core sweeps take (left-canonical, tall, 64+ columns) run
        there, the rest in the SIMT sweeps of the same call; "auto" does so
        when the tuning table measured the mixed form faster for the
        tensor-core gates' shape and count."""
        if not pairs:
            return
        precision = _native.PRECISION_PLAIN
        if self.precision in ("mixed", "auto"):
            d = self._qudit_dimension
            tc = []
            for p in pairs:
                m = int(self._site_list[p[1]].shape[0]) * d
                n = int(self._site_list[p[1] + 1].shape[2]) * d
                if p[3] and m >= n and n >= 64:
                    tc.append((m, n))
            if tc and (self.precision == "mixed" or autotune.lookup(
                    max(m for m, _ in tc), max(n for _, n in tc), d,
                    len(tc))["precision"] == "mixed"):
                precision = _native.PRECISION_MIXED
        self._run_pair_group(pairs, precision)

    def _run_pair_group(self, pairs, precision):
        """One mps_apply_2q_batch call for gates on disjoint adjacent pairs."""
        d = self._qudit_dimension
        dev = self._device
        njobs = len(pairs)
        if all(isinstance(p[0], torch.Tensor) for p in pairs):
            gates = torch.stack([p[0].reshape(d * d, d * d) for p in pairs]).to(
                dev, torch.complex64).contiguous()
        else:
            gates = torch.from_numpy(np.ascontiguousarray(
                np.stack([np.asarray(p[0]) for p in pairs]).astype(np.complex64))).to(dev)
        table = np.zeros(njobs, dtype=_native.JOB_DTYPE)
        outs = []
        max_m = max_n = 1
        rec = self.record_svals
        svals = disc = None
        status = torch.zeros(njobs, dtype=torch.int32, device=dev)
        if rec:
            rmax = max(min(int(self._sites[p[1]].shape[0]) * d, int(self._sites[p[1] + 1].shape[2]) * d)
                       for p in pairs)
            svals = torch.zeros((njobs, max(rmax, 1)), dtype=torch.float32, device=dev)
            disc = torch.zeros(njobs, dtype=torch.float64, device=dev)
        for q, (mat, left, k, lc) in enumerate(pairs):
            a, b = self._sites[left], self._sites[left + 1]
            chil, chim, chir = int(a.shape[0]), int(a.shape[2]), int(b.shape[2])
            a_out = torch.empty((chil, d, k), dtype=torch.complex64, device=dev)
            b_out = torch.empty((k, d, chir), dtype=torch.complex64, device=dev)
            outs.append((left, a_out, b_out))
            max_m = max(max_m, chil * d)
            max_n = max(max_n, chir * d)
            row = table[q]
            row["a"] = a.data_ptr()
            row["b"] = b.data_ptr()
            row["gate"] = gates[q].data_ptr()
            row["a_out"] = a_out.data_ptr() if a_out.numel() else 0
            row["b_out"] = b_out.data_ptr() if b_out.numel() else 0
            row["svals"] = svals[q].data_ptr() if rec else 0
            row["discarded"] = disc[q].data_ptr() if rec else 0
            row["status"] = status[q].data_ptr()
            row["chi_l"], row["chi_m"], row["chi_r"] = chil, chim, chir
            row["k"] = k
            row["keep_left_canonical"] = 1 if lc else 0
        jobs = torch.from_numpy(table.view(np.uint8)).to(dev)
        lib = self._lib()
        size_fn = (lib.mps_2q_workspace_bytes_mixed if precision == _native.PRECISION_MIXED
                   else lib.mps_2q_workspace_bytes)
        ws = _WS.get(dev, size_fn(njobs, max_m, max_n, d), "2q")
        timing = self.timing
        self.svd_params.precision = precision
        tuned = autotune.lookup(max_m, max_n, d, njobs) if self.autotune else autotune.DEFAULT
        self.svd_params.lq_off = tuned["lq_off"]
        self.svd_params.block_request = tuned["block_request"] if precision == 0 else 0
        if timing is not None:
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(torch.cuda.current_stream(dev))
        rc = lib.mps_apply_2q_batch(self._stream(), ctypes.c_void_p(jobs.data_ptr()), njobs,
                                    max_m, max_n, d, ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                                    ctypes.byref(self.svd_params))
        if timing is not None:
            ev1.record(torch.cuda.current_stream(dev))
            timing.append((njobs, max_m, max_n, self.svd_params.sweeps_out, ev0, ev1))
        _check_svd_rc(rc, self.on_unconverged)
        self._check_status(block=False)
        # the call returns before its last kernels: a NaN/Inf that first
        # appears after the first sweep only shows in the status words, read
        # here behind the call (no synchronisation)
        st_host = next((b for b in self._status_free if b.numel() >= njobs), None)
        if st_host is None:
            st_host = torch.empty(max(njobs, 64), dtype=torch.int32, pin_memory=True)
        else:
            self._status_free.remove(st_host)
        st_host[njobs:].zero_()
        st_host[:njobs].copy_(status, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(dev))
        self._status_pending.append((st_host, ev))
        for left, a_out, b_out in outs:
            self._sites[left] = a_out
            self._version += 1
            self._sites[left + 1] = b_out
        if rec:
            sv = svals.cpu().numpy()
            dc = disc.cpu().numpy()
            for q, (mat, left, k, lc) in enumerate(pairs):
                a_out = outs[q][1]
                r = min(int(a_out.shape[0]) * d, int(outs[q][2].shape[2]) * d)
                self.svals_history.append((sv[q, :r].astype(np.float64), k, float(dc[q])))

    def move_node_from_left_to_right(self, current_node_index: int, final_node_index: int,
                                     **kwargs) -> None:
        """Chain of SWAPs (core.py:1163-1190)."""
        if current_node_index > final_node_index:
            raise ValueError("current_node_index should be smaller than final_node_index.")
        if current_node_index < 0:
            raise ValueError("current_node_index out of range.")
        if final_node_index >= self._nqudits:
            raise ValueError("final_node_index out of range.")
        while current_node_index < final_node_index:
            self.swap(current_node_index, current_node_index + 1, **kwargs)
            current_node_index += 1

    def move_node_from_right_to_left(self, current_node_index: int, final_node_index: int,
                                     **kwargs) -> None:
        """Chain of SWAPs (core.py:1192-1219)."""
        if current_node_index < final_node_index:
            raise ValueError("current_node_index should be larger than final_node_index.")
        if current_node_index > self._nqudits:
            raise ValueError("current_node_index out of range.")
        if final_node_index < 0:
            raise ValueError("final_node_index out of range.")
        while current_node_index > final_node_index:
            self.swap(current_node_index - 1, current_node_index, **kwargs)
            current_node_index -= 1

    # -- operation lists ---------------------------------------------------
    def apply(self, operations, **kwargs) -> None:
        """Applies operations in order (core.py:1221-1276), each through
        apply_one_qudit_gate / apply_two_qudit_gate: two-qudit gates on
        disjoint adjacent pairs join the state's queue and run as one batched
        launch, so the result equals in-order application.  Consecutive
        two-qudit operations whose site ranges (all sites from the lower to
        the higher index, which a non-adjacent gate's SWAP chains cross) are
        disjoint are interleaved step by step (_two_qudit_steps), so that
        the k-th SWAP of every chain joins one launch; each chain keeps its
        own order and touches no other chain's sites, so the result is the
        in-order one.  An operation that fails validation first lets the
        operations before it run, as in-order application would.  With
        track_norms every operation runs on its own (the norm history is
        per operation)."""
        try:
            operations = iter(operations)
        except TypeError:
            operations = (operations,)
        group = []                        # step lists of two-qudit operations
        used = set()                      # the sites their ranges cover

        def run_group():
            chains = list(group)
            group.clear()
            used.clear()
            for t in range(max((len(c) for c in chains), default=0)):
                for c in chains:
                    if t < len(c):
                        c[t]()

        try:
            for op in operations:
                if not isinstance(op, MPSOperation):
                    raise TypeError("Argument operation should be of type MPSOperation but is "
                                    f"of type {type(op)}.")
                if not op.is_valid():
                    raise ValueError("Input MPS Operation is not valid.")
                if op.is_single_qudit_operation():
                    run_group()
                    (i,) = op.qudit_indices
                    self.apply_one_qudit_gate(op.node(copy=False), i, **kwargs)
                elif op.is_two_qudit_operation():
                    i, j = op.qudit_indices
                    if self.track_norms:
                        run_group()
                        self.apply_two_qudit_gate(op.node(copy=False), i, j, **kwargs)
                        continue
                    node = op.node(copy=False)
                    self._check_two_qudit(node, i, j)
                    span = set(range(min(i, j), max(i, j) + 1))
                    if span & used:
                        run_group()
                    group.append(self._two_qudit_steps(node, i, j, kwargs))
                    used.update(span)
                else:
                    raise ValueError(
                        "Only one-qudit and two-qudit gates are supported. To apply a gate on "
                        "three or more qudits, the gate must be compiled into a sequence of one- "
                        "and two-qudit gates.")
        except BaseException:
            run_group()
            raise
        run_group()

    def _two_qudit_steps(self, gate, i: int, j: int, kwargs) -> list:
        """apply_two_qudit_gate(gate, i, j) as its sequence of adjacent steps
        (core.py:1034-1058): SWAPs carrying the lower site up to the higher
        one's neighbour, the gate there (in the caller's orientation), SWAPs
        back."""
        lo, hi = min(i, j), max(i, j)
        steps = [lambda a=a: self.swap(a, a + 1, **kwargs) for a in range(lo, hi - 1)]
        if i < j:
            steps.append(lambda: self.apply_two_qudit_gate(gate, hi - 1, hi, **kwargs))
        else:
            steps.append(lambda: self.apply_two_qudit_gate(gate, hi, hi - 1, **kwargs))
        steps += [lambda a=a: self.swap(a, a + 1, **kwargs) for a in range(hi - 2, lo - 1, -1)]
        return steps

    def apply_layer(self, one_qudit: Optional[np.ndarray], pair_left: Sequence[int],
                    two_qudit: Optional[np.ndarray], **kwargs) -> None:
        """One brickwork layer: ``one_qudit[i]`` (d x d) on every site i, then
        ``two_qudit[p]`` (d^2 x d^2) on (pair_left[p], pair_left[p] + 1), the
        pairs disjoint -- the same result as applying the gates one by one."""
        self._flush()
        if one_qudit is not None:
            self._apply_one_qudit_layer(one_qudit)
        if two_qudit is None or len(pair_left) == 0:
            return
        if not self.is_valid():
            raise ValueError("MPS is not valid.")
        used = set()
        pairs = []
        for p, i in enumerate(pair_left):
            i = int(i)
            if i in used or i + 1 in used:
                raise ValueError("apply_layer pairs must be disjoint")
            used.update((i, i + 1))
            pairs.append(self._prepare_pair(np.asarray(two_qudit[p]).reshape((self._qudit_dimension,) * 4),
                                            i, i + 1, kwargs, checked=True))
        if self.track_norms:
            for pr in pairs:
                self._run_pairs([pr])
                self._norms.append(self.norm())
        else:
            self._run_pairs(pairs)

    def apply_layer_resident(self, one_qudit_dev, pair_left: Sequence[int], two_qudit_dev,
                             maxsvals: Optional[int] = None, keep_left_canonical: bool = True) -> None:
        """``apply_layer`` for gates already on the device (torch complex64:
        one_qudit_dev (n, d, d), two_qudit_dev (p, d^2, d^2)).  Skips the
        host-side unitarity and edge checks; shapes are still validated."""
        self._flush()
        d = self._qudit_dimension
        if one_qudit_dev is not None:
            if tuple(one_qudit_dev.shape) != (self._nqudits, d, d):
                raise ValueError("one_qudit_dev must have shape (nqudits, d, d)")
            table = np.zeros(self._nqudits, dtype=_native.JOB1_DTYPE)
            for i, site in enumerate(self._sites):
                table[i]["site"] = site.data_ptr()
                table[i]["gate"] = one_qudit_dev[i].data_ptr()
                table[i]["chi_l"], table[i]["chi_r"] = int(site.shape[0]), int(site.shape[2])
            jt = torch.from_numpy(table.view(np.uint8)).to(self._device)
            _native.check(self._lib().mps_apply_1q_batch(
                self._stream(), ctypes.c_void_p(jt.data_ptr()), self._nqudits, d))
        if two_qudit_dev is None or len(pair_left) == 0:
            return
        used = set()
        pairs = []
        for p, i in enumerate(pair_left):
            i = int(i)
            if i in used or i + 1 in used or not (0 <= i < self._nqudits - 1):
                raise ValueError("apply_layer_resident pairs must be disjoint and in range")
            used.update((i, i + 1))
            a, b = self._sites[i], self._sites[i + 1]
            k = kept_count(maxsvals, min(int(a.shape[0]) * d, int(b.shape[2]) * d))
            pairs.append((two_qudit_dev[p], i, k, bool(keep_left_canonical)))
        self._run_pairs(pairs)

    # -- shorthands (core.py:1278-1380) --------------------------------------
    def x(self, index: int) -> None:
        if index == -1:
            self.apply_one_qudit_gate_to_all(xgate())
        else:
            self.apply_one_qudit_gate(xgate(), index)

    def h(self, index: int) -> None:
        if index == -1:
            self.apply_one_qudit_gate_to_all(hgate())
        else:
            self.apply_one_qudit_gate(hgate(), index)

    def r(self, index, seed: Optional[int] = None, angle_scale: float = 1.0) -> None:
        if index == -1:
            for i in range(self._nqudits):
                self.apply_one_qudit_gate(rgate(seed, angle_scale), i)
        else:
            self.apply_one_qudit_gate(rgate(seed, angle_scale), index)

    def cnot(self, a: int, b: int, **kwargs) -> None:
        self.apply_two_qudit_gate(cnot(), a, b, **kwargs)

    def haar_random(self, qudit1_index: int, qudit2_index: int, **kwargs) -> None:
        gate = haar_random_unitary(nqudits=2, qudit_dimension=self._qudit_dimension)
        self.apply_two_qudit_gate(gate, qudit1_index, qudit2_index, **kwargs)

    def sweep_haar_random_left_to_right(self, **kwargs) -> None:
        for i in range(0, self._nqudits - 1, 2):
            self.haar_random(i, i + 1, keep_left_canonical=True, **kwargs)

    def sweep_haar_random_right_to_left(self, **kwargs) -> None:
        for i in range(self._nqudits - 2, 0, -2):
            self.haar_random(i - 1, i, keep_left_canonical=False, **kwargs)

    def sweep_cnots_left_to_right(self, **kwargs) -> None:
        for i in range(0, self._nqudits - 1, 2):
            self.cnot(i, i + 1, keep_left_canonical=True, **kwargs)

    def sweep_cnots_right_to_left(self, **kwargs) -> None:
        for i in range(self._nqudits - 2, 0, -2):
            self.cnot(i - 1, i, keep_left_canonical=False, **kwargs)

    def swap(self, a: int, b: int, **kwargs) -> None:
        if b < a:
            a, b = b, a
        self.apply_two_qudit_gate(swap(), a, b, **kwargs)

    # -- copies / comparison ---------------------------------------------
    def copy(self) -> "MPS":
        return self.__copy__()

    def __copy__(self):
        sites = self._sites                   # runs queued gates first
        new = MPS.__new__(MPS)
        new.__dict__.update(self.__dict__)
        new._pending = []
        new._pending_sites = set()
        new._pending_1q = []
        new._pending_1q_sites = set()
        new._site_list = [t.clone() for t in sites]
        new._norms = list(self._norms)
        new.svals_history = list(self.svals_history)
        new.svd_params = _native.SvdParams(self.svd_params.max_sweeps, self.svd_params.tol, 0, 0,
                                           self.svd_params.wait_limit, 0,
                                           self.svd_params.precision, self.svd_params.lq_off,
                                           self.svd_params.block_request)
        return new

    def __str__(self):
        return "----".join(f"{self._prefix}{i}{tuple(t.shape)}" for i, t in enumerate(self._sites))

    def __eq__(self, other):
        if not isinstance(other, MPS):
            return False
        if self is other:
            return True
        if not self.is_valid():
            raise ValueError("MPS is invalid and cannot be compared to another MPS.")
        if not other.is_valid():
            raise ValueError("Other MPS is invalid.")
        if other._qudit_dimension != self._qudit_dimension or other._nqudits != self._nqudits:
            return False
        for a, b in zip(self._sites, other._sites):
            if tuple(a.shape) != tuple(b.shape):
                return False
            if not np.allclose(a.cpu().numpy(), b.cpu().numpy()):
                return False
        return True

    def __ne__(self, other):
        return not self.__eq__(other)

    __hash__ = None
