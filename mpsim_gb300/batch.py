"""Many independent circuits advanced together (the multi-circuit form).

``MPSBatch`` holds a list of ``MPS`` states (any qudit counts, one qudit
dimension) and applies one layer of each circuit per ``step``: every one-qudit
gate of every circuit in one ``mps_apply_1q_batch`` launch, and every
two-qudit gate of every circuit in one ``mps_apply_2q_batch`` call per slot
size class (jobs are grouped by the padded length of their merged matrix so a
few large gates do not inflate the scratch slots of many small ones).  Each
circuit's result is exactly what applying its gates one by one gives: a
layer's two-qudit gates act on disjoint pairs, and different circuits share
nothing.
"""

from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native
from .core import MPS, _WS, kept_count

# padded merged-matrix lengths of the two-qudit kernel's slot classes
_CLASSES = (64, 128, 256, 512, 576, 1024, 1792)


def _slot_class(m: int, n: int) -> int:
    L = max(m, n, 1)
    for c in _CLASSES:
        if L <= c:
            return c
    raise ValueError(f"merged matrix of {L} rows is beyond this build's two-qudit kernel")


class MPSBatch:
    def __init__(self, states: Sequence[MPS]):
        if not states:
            raise ValueError("MPSBatch needs at least one state")
        d = states[0].qudit_dimension
        if any(s.qudit_dimension != d for s in states):
            raise ValueError("all states of a batch must share the qudit dimension")
        dev = states[0].device
        if any(s.device != dev for s in states):
            raise ValueError("all states of a batch must live on one device")
        self.states = list(states)
        self.d = d
        self.device = dev
        self.svd_params = _native.SvdParams()
        self.sweeps = []

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def step(self, layers: Sequence[Optional[tuple]], maxsvals: Sequence[Optional[int]],
             keep_left_canonical: bool = True) -> int:
        """Apply ``layers[c]`` = (one_q (n,d,d), pair_left, two_q (p,d^2,d^2)) to
        state c (None skips it) with truncation ``maxsvals[c]``.  Returns the
        number of two-qudit gates applied."""
        if len(layers) != len(self.states) or len(maxsvals) != len(self.states):
            raise ValueError("one layer and one maxsvals per state")
        lib = _native.load()
        d, dev = self.d, self.device
        # one-qudit gates: one launch over every site of every active circuit
        ones, sites1 = [], []
        for st, lay in zip(self.states, layers):
            if lay is None or lay[0] is None:
                continue
            one = np.asarray(lay[0])
            if one.shape != (st.nqudits, d, d):
                raise ValueError("one-qudit gates must have shape (nqudits, d, d)")
            ones.append(one)
            sites1.extend(st._sites)
        if sites1:
            g1 = torch.from_numpy(np.ascontiguousarray(
                np.concatenate(ones).astype(np.complex64))).to(dev)
            t1 = np.zeros(len(sites1), dtype=_native.JOB1_DTYPE)
            for q, site in enumerate(sites1):
                t1[q]["site"] = site.data_ptr()
                t1[q]["gate"] = g1[q].data_ptr()
                t1[q]["chi_l"], t1[q]["chi_r"] = int(site.shape[0]), int(site.shape[2])
            for lo in range(0, len(sites1), 65535):
                part = t1[lo:lo + 65535]
                jt = torch.from_numpy(part.view(np.uint8).copy()).to(dev)
                _native.check(lib.mps_apply_1q_batch(self._stream(), ctypes.c_void_p(jt.data_ptr()),
                                                     len(part), d))
        # two-qudit gates: one call per slot class
        buckets = {}
        gates, owners = [], []
        for c, (st, lay) in enumerate(zip(self.states, layers)):
            if lay is None or lay[2] is None or len(lay[1]) == 0:
                continue
            used = set()
            for p, i in enumerate(lay[1]):
                i = int(i)
                if i in used or i + 1 in used or not (0 <= i < st.nqudits - 1):
                    raise ValueError("a layer's pairs must be disjoint and in range")
                used.update((i, i + 1))
                a, b = st._sites[i], st._sites[i + 1]
                m, n = int(a.shape[0]) * d, int(b.shape[2]) * d
                k = kept_count(maxsvals[c], min(m, n))
                gates.append(np.asarray(lay[2][p]).reshape(d * d, d * d))
                owners.append((c, i, k, m, n))
        if not owners:
            return 0
        g2 = torch.from_numpy(np.ascontiguousarray(np.stack(gates).astype(np.complex64))).to(dev)
        for q, own in enumerate(owners):
            buckets.setdefault(_slot_class(own[3], own[4]), []).append(q)
        for cls in sorted(buckets):
            idxs = buckets[cls]
            for lo in range(0, len(idxs), 65535):
                self._run_class(lib, g2, [owners[q] for q in idxs[lo:lo + 65535]],
                                idxs[lo:lo + 65535], keep_left_canonical)
        return len(owners)

    def _run_class(self, lib, g2, owners, gidx, lc):
        d, dev = self.d, self.device
        table = np.zeros(len(owners), dtype=_native.JOB_DTYPE)
        outs = []
        max_m = max_n = 1
        status = torch.zeros(len(owners), dtype=torch.int32, device=dev)
        for q, ((c, i, k, m, n), gq) in enumerate(zip(owners, gidx)):
            st = self.states[c]
            a, b = st._sites[i], st._sites[i + 1]
            chil, chim, chir = int(a.shape[0]), int(a.shape[2]), int(b.shape[2])
            a_out = torch.empty((chil, d, k), dtype=torch.complex64, device=dev)
            b_out = torch.empty((k, d, chir), dtype=torch.complex64, device=dev)
            outs.append((c, i, a_out, b_out))
            row = table[q]
            row["a"], row["b"], row["gate"] = a.data_ptr(), b.data_ptr(), g2[gq].data_ptr()
            row["a_out"] = a_out.data_ptr() if a_out.numel() else 0
            row["b_out"] = b_out.data_ptr() if b_out.numel() else 0
            row["status"] = status[q].data_ptr()
            row["chi_l"], row["chi_m"], row["chi_r"], row["k"] = chil, chim, chir, k
            row["keep_left_canonical"] = 1 if lc else 0
            max_m, max_n = max(max_m, m), max(max_n, n)
        jobs = torch.from_numpy(table.view(np.uint8)).to(dev)
        nbytes = lib.mps_2q_workspace_bytes(len(owners), max_m, max_n, d)
        ws = _WS.get(dev, nbytes, "batch2q")
        rc = lib.mps_apply_2q_batch(self._stream(), ctypes.c_void_p(jobs.data_ptr()), len(owners),
                                    max_m, max_n, d, ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                                    ctypes.byref(self.svd_params))
        if rc not in (_native.MPS_OK, _native.MPS_ERR_NOT_CONVERGED):
            raise _native.NativeError(rc, _native.last_error())
        self.sweeps.append(self.svd_params.sweeps_out)
        for c, i, a_out, b_out in outs:
            self.states[c]._sites[i] = a_out
            self.states[c]._sites[i + 1] = b_out
            self.states[c]._version += 1


def run_circuits(circuits, device=None) -> List[MPS]:
    """Simulate seeded ``BrickworkCircuit``s together; returns the final states."""
    states = [MPS(c.nqudits, c.d) for c in circuits]
    batch = MPSBatch(states)
    depth = max(c.depth for c in circuits)
    for t in range(depth):
        layers = [(c.layers[t].one_q, c.layers[t].pair_left, c.layers[t].two_q)
                  if t < c.depth else None for c in circuits]
        batch.step(layers, [c.maxsvals for c in circuits])
    return states
