"""Whole circuits planned once and replayed: the batched form and the CUDA-graph
layer step.

``CircuitPlan`` takes one or many seeded brickwork circuits (any qudit counts
and depths, one qudit dimension) and plans every launch before the first one:
the bond dimension after every two-qudit gate is ``min(maxsvals, min(m, n))``
(mpsim/core.py:1110-1137; no tolerance-based truncation), so every site shape
of every layer is known on the host.  It then

* puts every gate matrix on the device in one copy;
* gives each (circuit, site) two buffers of the largest size that site ever
  has, plus the product state, in one arena: a two-qudit gate reads the
  current buffers of its sites and writes the other ones (a one-qudit gate
  works in place), so the arena is twice the largest state, not the sum of
  all intermediate states;
* builds every job table (``mps_1q_job`` / ``mps_2q_job``) in NumPy and copies
  all of them to the device at once;
* groups each global layer's jobs into calls: one ``mps_apply_1q_batch`` for
  every one-qudit gate of every circuit in the layer, and one
  ``mps_apply_2q_batch`` per slot-size class for the two-qudit gates, so a
  few large gates do not inflate the scratch slots of many small ones (with
  precision="mixed" each such call is MPS_PRECISION_MIXED: its tensor-core
  gates and its other gates share the call).  Circuits shorter than the deepest one simply drop out of the later
  layers.

``run()`` then issues only library calls -- no host work per gate, no copies
-- and ``capture()`` records the same calls as one CUDA graph (the two-qudit
call runs a fixed number of sweeps under capture, converged jobs returning at
once, and reports through its per-job status words; ``replay()`` checks
them).  Each circuit's result equals applying its gates one by one:
``apply_layer``'s gates act on disjoint pairs, and circuits share nothing.
"""

from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native
from . import autotune as _autotune
from .core import MPS, kept_count

# padded merged-matrix lengths of the two-qudit kernel's slot classes
SLOT_CLASSES = (64, 128, 256, 512, 576, 1024, 1792)
_ALIGN = 256
_CHUNK = 65535                      # jobs per call (grid limit of the kernels)


def slot_class(m: int, n: int) -> int:
    L = max(m, n, 1)
    for c in SLOT_CLASSES:
        if L <= c:
            return c
    raise ValueError(f"merged matrix of {L} rows is beyond this build's two-qudit kernel")


def _tc_eligible(m: int, n: int, lc: bool) -> bool:
    """The gates MPS_PRECISION_MIXED takes: left-canonical, tall, 64+ columns."""
    return lc and m >= n and n >= 64


class CircuitPlan:
    """See the module docstring.  ``circuits``: objects with ``nqudits``,
    ``d``, ``depth``, ``maxsvals`` and ``layers`` (each with ``one_q`` (n, d,
    d), ``pair_left`` and ``two_q`` (p, d^2, d^2)), e.g. ``circuits.brickwork``."""

    def __init__(self, circuits: Sequence, device=None, precision: str = "plain",
                 keep_left_canonical: bool = True, max_sweeps: int = 40, autotune: bool = True):
        if not circuits:
            raise ValueError("CircuitPlan needs at least one circuit")
        if precision not in ("plain", "mixed", "auto"):
            raise ValueError("precision must be 'plain', 'mixed' or 'auto'")
        d = int(circuits[0].d)
        if any(int(c.d) != d for c in circuits):
            raise ValueError("all circuits of a plan must share the qudit dimension")
        if device is None:
            if not torch.cuda.is_available():
                raise RuntimeError("CircuitPlan runs on a CUDA GPU only (no CPU fallback)")
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self.d = d
        self.circuits = list(circuits)
        self.precision = precision
        self.max_sweeps = int(max_sweeps)
        lc = bool(keep_left_canonical)
        self.lib = _native.load()
        self.graph = None

        # ---- gates: one upload -----------------------------------------
        ones, twos, one_base, two_base = [], [], [], []
        n1 = n2 = 0
        for c in self.circuits:
            ob, tb = [], []
            for lay in c.layers:
                o = np.asarray(lay.one_q, dtype=np.complex64).reshape(-1, d, d)
                t = np.asarray(lay.two_q, dtype=np.complex64).reshape(-1, d * d, d * d)
                ones.append(o)
                twos.append(t)
                ob.append(n1)
                tb.append(n2)
                n1 += o.shape[0]
                n2 += t.shape[0]
            one_base.append(ob)
            two_base.append(tb)
        self.g1 = torch.from_numpy(np.ascontiguousarray(np.concatenate(ones))).to(self.device)
        self.g2 = torch.from_numpy(np.ascontiguousarray(np.concatenate(twos))).to(self.device)
        g1p, g2p = self.g1.data_ptr(), self.g2.data_ptr()
        s1, s2 = d * d * 8, d ** 4 * 8

        # ---- shapes: bond dimensions after every gate --------------------
        # per circuit: bonds[i] between site i and i+1; track the largest
        # size of every site over the circuit
        bonds = [[1] * (c.nqudits - 1) for c in self.circuits]
        maxsite = [[d] * c.nqudits for c in self.circuits]   # complex elements
        depth = max(c.depth for c in self.circuits)
        events = []     # per layer: list of (c, i, pair, chil, chim, chir, k)
        for t in range(depth):
            ev = []
            for ci, c in enumerate(self.circuits):
                if t >= c.depth:
                    continue
                b = bonds[ci]
                for p, i in enumerate(c.layers[t].pair_left):
                    i = int(i)
                    chil = b[i - 1] if i > 0 else 1
                    chim = b[i]
                    chir = b[i + 1] if i + 1 < c.nqudits - 1 else 1
                    k = kept_count(c.maxsvals, min(chil * d, chir * d))
                    b[i] = k
                    ev.append((ci, i, p, chil, chim, chir, k))
                    maxsite[ci][i] = max(maxsite[ci][i], chil * d * k)
                    maxsite[ci][i + 1] = max(maxsite[ci][i + 1], k * d * chir)
            events.append(ev)

        # ---- arena: product state + two buffers per site -----------------
        # the product state of every circuit first (contiguous: one reset copy)
        off = 0
        start_off, buf_off = [], []
        for c in self.circuits:
            so = []
            for i in range(c.nqudits):
                so.append(off)
                off += -(-d * 8 // _ALIGN) * _ALIGN
            start_off.append(so)
        self._nstart = max(off, _ALIGN)
        for ci, c in enumerate(self.circuits):
            bo = []
            for i in range(c.nqudits):
                nb = -(-maxsite[ci][i] * 8 // _ALIGN) * _ALIGN
                bo.append((off, off + nb))
                off += 2 * nb
            buf_off.append(bo)
        self.arena = torch.zeros(max(off, _ALIGN), dtype=torch.uint8, device=self.device)
        base = self.arena.data_ptr()
        prist = np.zeros(self._nstart // 8, dtype=np.complex64)
        for ci, c in enumerate(self.circuits):
            for i in range(c.nqudits):
                prist[start_off[ci][i] // 8] = 1.0          # |0> on every site
        self._pristine = torch.from_numpy(prist.view(np.uint8)).to(self.device)

        # ---- job tables and calls ----------------------------------------
        cur = [[(start_off[ci][i], (1, 1)) for i in range(c.nqudits)]
               for ci, c in enumerate(self.circuits)]            # (offset, (chil, chir))
        which = [[0] * c.nqudits for c in self.circuits]          # next buffer to write
        rows1, rows2 = [], []
        calls = []
        status_n = 0
        for t in range(depth):
            # one-qudit gates of every active circuit
            lo = len(rows1)
            for ci, c in enumerate(self.circuits):
                if t >= c.depth:
                    continue
                gb = one_base[ci][t]
                for i in range(c.nqudits):
                    o, (cl, cr) = cur[ci][i]
                    rows1.append((base + o, g1p + (gb + i) * s1, cl, cr))
            for a in range(lo, len(rows1), _CHUNK):
                calls.append(("1q", a, min(_CHUNK, len(rows1) - a)))
            # two-qudit gates, grouped by slot class
            groups = {}
            for ci, i, p, chil, chim, chir, k in events[t]:
                m, n = chil * d, chir * d
                elig = precision in ("mixed", "auto") and _tc_eligible(m, n, lc)
                oa, ob = cur[ci][i][0], cur[ci][i + 1][0]
                wa, wb = which[ci][i], which[ci][i + 1]
                na, nbo = buf_off[ci][i][wa], buf_off[ci][i + 1][wb]
                which[ci][i], which[ci][i + 1] = 1 - wa, 1 - wb
                cur[ci][i] = (na, (chil, k))
                cur[ci][i + 1] = (nbo, (k, chir))
                row = (base + oa, base + ob, g2p + (two_base[ci][t] + p) * s2,
                       base + na if chil * k else 0, base + nbo if k * chir else 0, 0, 0,
                       status_n, chil, chim, chir, k, 1 if lc else 0, 0)
                status_n += 1
                groups.setdefault(slot_class(m, n), []).append((row, m, n, elig))
            for _cls, items in sorted(groups.items()):
                for a in range(0, len(items), _CHUNK):
                    part = items[a:a + _CHUNK]
                    # one call per slot class: MPS_PRECISION_MIXED sends its
                    # tensor-core gates to the tensor-core sweeps and the rest
                    # to the SIMT ones ("auto": where the tuning table found
                    # the mixed form faster for those gates)
                    tcs = [(m, n) for _, m, n, e in part if e]
                    prec = _native.PRECISION_PLAIN
                    if tcs and (precision == "mixed" or _autotune.lookup(
                            max(m for m, _ in tcs), max(n for _, n in tcs), d,
                            len(tcs))["precision"] == "mixed"):
                        prec = _native.PRECISION_MIXED
                    lo2 = len(rows2)
                    rows2.extend(r for r, _, _, _ in part)
                    mm, nn = max(m for _, m, _, _ in part), max(n for _, _, n, _ in part)
                    tuned = (_autotune.lookup(mm, nn, d, len(part)) if autotune
                             else _autotune.DEFAULT)
                    calls.append(("2q", lo2, len(part), mm, nn, prec, tuned["lq_off"],
                                  tuned["block_request"] if prec == _native.PRECISION_PLAIN else 0))
        self.n_two_qudit_gates = status_n
        self.status = torch.zeros(max(status_n, 1), dtype=torch.int32, device=self.device)
        sp = self.status.data_ptr()
        t1 = np.zeros(len(rows1), dtype=_native.JOB1_DTYPE)
        if rows1:
            r1 = np.array(rows1, dtype=np.int64)
            t1["site"], t1["gate"] = r1[:, 0].astype(np.uint64), r1[:, 1].astype(np.uint64)
            t1["chi_l"], t1["chi_r"] = r1[:, 2], r1[:, 3]
        t2 = np.zeros(len(rows2), dtype=_native.JOB_DTYPE)
        if rows2:
            r2 = np.array(rows2, dtype=np.int64)
            for f, col in (("a", 0), ("b", 1), ("gate", 2), ("a_out", 3), ("b_out", 4)):
                t2[f] = r2[:, col].astype(np.uint64)
            t2["status"] = (sp + 4 * r2[:, 7]).astype(np.uint64)
            for f, col in (("chi_l", 8), ("chi_m", 9), ("chi_r", 10), ("k", 11),
                           ("keep_left_canonical", 12)):
                t2[f] = r2[:, col]
        self.t1 = torch.from_numpy(t1.view(np.uint8).copy()).to(self.device)
        self.t2 = torch.from_numpy(t2.view(np.uint8).copy()).to(self.device)
        self.calls = calls
        ws = 1
        for cl in calls:
            if cl[0] == "2q":
                size_fn = (self.lib.mps_2q_workspace_bytes_mixed
                           if cl[5] == _native.PRECISION_MIXED else self.lib.mps_2q_workspace_bytes)
                ws = max(ws, int(size_fn(cl[2], cl[3], cl[4], d)))
        self.workspace = torch.empty(ws, dtype=torch.uint8, device=self.device)
        self._final = [[(o, shp) for (o, shp) in cur[ci]] for ci in range(len(self.circuits))]
        self._params = _native.SvdParams()
        # sweeps each two-qudit call took in the last eager run: a captured
        # call runs exactly its budget (converged jobs return at once from
        # the extra sweeps), and a fixed plan repeats the same sweeps on every
        # run, so the budget is the observed count plus a margin
        self.sweeps = [None] * len(calls)
        self.sweep_margin = 2

    # -- execution ---------------------------------------------------------
    def _reset(self):
        """Product state |0...0> in the start buffers (one device copy)."""
        self.arena[: self._nstart].copy_(self._pristine[: self._nstart])

    def run(self) -> None:
        """Issues every call of the plan on the current stream."""
        lib, d = self.lib, self.d
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        self._reset()
        j1, j2 = self.t1.data_ptr(), self.t2.data_ptr()
        p = self._params
        capturing = torch.cuda.is_current_stream_capturing()
        for ci, cl in enumerate(self.calls):
            if cl[0] == "1q":
                _native.check(lib.mps_apply_1q_batch(
                    stream, ctypes.c_void_p(j1 + cl[1] * _native.JOB1_DTYPE.itemsize), cl[2], d))
                continue
            _, lo, n, max_m, max_n, prec, lq_off, block = cl
            p.precision = prec
            p.lq_off, p.block_request = lq_off, block
            p.max_sweeps = self.max_sweeps
            if capturing and self.sweeps[ci] is not None:
                p.max_sweeps = min(self.max_sweeps, self.sweeps[ci] + self.sweep_margin)
            rc = lib.mps_apply_2q_batch(
                stream, ctypes.c_void_p(j2 + lo * _native.JOB_DTYPE.itemsize), n, max_m, max_n,
                d, ctypes.c_void_p(self.workspace.data_ptr()), self.workspace.numel(),
                ctypes.byref(p))
            # (under capture the call reports through the status words only)
            if rc != _native.MPS_OK:
                raise _native.NativeError(rc, _native.last_error())
            if not capturing:
                self.sweeps[ci] = int(p.sweeps_out)

    def capture(self) -> None:
        """Records run() as one CUDA graph, after one eager run that sets up the
        library's per-device state and records each call's sweep count (the
        captured budget is that count plus ``sweep_margin``; a replay that ever
        needed more reports MPS_STATUS_NOT_CONVERGED through the status words,
        which ``replay`` checks)."""
        self.run()
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.run()
        torch.cuda.synchronize(self.device)

    def replay(self, check: bool = True) -> None:
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()
        if check:
            self.check_status()

    def check_status(self) -> None:
        """Raises if a two-qudit job of the last run reported a problem: a
        captured call can report only through these words."""
        st = self.status[: max(self.n_two_qudit_gates, 1)].cpu().numpy()
        bad = np.flatnonzero(st)
        if bad.size:
            bits = int(np.bitwise_or.reduce(st[bad]))
            if bits & _native.STATUS_NONFINITE:
                code = _native.MPS_ERR_NONFINITE
            elif bits & _native.STATUS_TIMEOUT:
                code = _native.MPS_ERR_TIMEOUT
            else:
                code = _native.MPS_ERR_NOT_CONVERGED
            raise _native.NativeError(code, f"{bad.size} two-qudit gate(s) reported status bits "
                                            f"{bits:#x} (1: not converged, 2: NaN/Inf, 4: timeout)")

    # -- results -------------------------------------------------------------
    def final_sites(self, index: int) -> List[torch.Tensor]:
        """Device views of circuit ``index``'s final site tensors (rewritten by
        every run or replay)."""
        d = self.d
        out = []
        for o, (cl, cr) in self._final[index]:
            nbytes = cl * d * cr * 8
            out.append(self.arena[o:o + nbytes].view(torch.complex64).view(cl, d, cr))
        return out

    def state(self, index: int, precision: Optional[str] = None) -> MPS:
        """Circuit ``index``'s final state as an MPS sharing the plan's
        buffers (a later run or replay overwrites it; copy() to keep it)."""
        c = self.circuits[index]
        return MPS.from_sites(self.final_sites(index), c.d,
                              precision=precision or self.precision)
