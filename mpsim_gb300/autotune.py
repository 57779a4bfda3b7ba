"""Autotuner of the two-qudit call, keyed on (theta shape, d, batch).

The choices it makes per call (fields of ``mps_svd_params``):

* ``lq_off``        -- run the Jacobi sweeps on theta itself instead of its L
  factor (the LQ factorisation costs panels on a few SMs; the sweeps it saves
  depend on the shape);
* ``block_request`` -- 16- or 8-column blocks in the plain sweep kernel for
  512 / 576-row slots (fewer registers and more resident CTAs against more
  rounds per sweep);
* ``precision``     -- for ``MPS(precision="auto")``: the plain FP32 sweeps or
  the tensor-core block sweeps, whichever is faster for that shape and batch.

``tune()`` times every candidate on seeded random jobs of each shape
(synthetic sites with the workloads' bond dimensions, Haar gates), after a
correctness guard (singular values equal to the default configuration's
within 1e-4 s_0), and writes the winners to a JSON table; ``lookup()`` reads
it.  The committed table ``tuning/gb300.json`` was measured on a GB300 with
``python -m mpsim_gb300.autotune``; shapes missing from it take the defaults.
Batch sizes are bucketed (<= 8, <= 64, more): a layer of one 64-qubit circuit
is 32 jobs, a batched layer of many circuits thousands.
"""

from __future__ import annotations

import ctypes
import json
import os
import time
from typing import Dict, Optional

import numpy as np

from . import _native

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "tuning", "gb300.json")
# Batch-size buckets of the table: a call of njobs jobs takes the entry of the
# smallest bucket >= njobs, which is measured at the smallest batch the bucket
# covers (the previous bound + 1).  The mixed form's advantage grows with the
# batch (a visit's latency bounds it, the plain form is bound by its work), so
# a bucket takes the mixed form only where it wins for every batch it covers.
BUCKETS = (8, 16, 32, 64, 128, 256, 1 << 30)
TUNE_BATCHES = (1,) + tuple(b + 1 for b in BUCKETS[:-1])
DEFAULT = {"lq_off": 0, "block_request": 0, "precision": "plain"}

_table = None


def bucket(njobs: int) -> int:
    for b in BUCKETS:
        if njobs <= b:
            return b
    return BUCKETS[-1]


def key(m: int, n: int, d: int, njobs: int) -> str:
    return f"d{d}_m{m}_n{n}_b{min(bucket(njobs), 1 << 20)}"


def load_table(path: str = TABLE_PATH) -> Dict:
    global _table
    if _table is None or path != TABLE_PATH:
        t = {}
        if os.path.exists(path):
            with open(path) as f:
                t = json.load(f).get("entries", {})
        if path != TABLE_PATH:
            return t
        _table = t
    return _table


def lookup(m: int, n: int, d: int, njobs: int, table: Optional[Dict] = None) -> Dict:
    """The tuned settings for a call whose largest theta is m x n (defaults
    where the table has no entry).  Keys: lq_off, block_request, precision
    (the faster of "plain" and "mixed" for this shape)."""
    t = load_table() if table is None else table
    e = t.get(key(m, n, d, njobs))
    out = dict(DEFAULT)
    if e:
        out.update({k: e[k] for k in DEFAULT if k in e})
    return out


def candidates(m: int, n: int, lc: bool = True):
    """(precision, lq_off, block_request) triples valid for this shape."""
    L = max(m, n)
    out = []
    for lq_off in (0, 1):
        out.append(("plain", lq_off, 0))
        if 256 < L <= 576:
            out.append(("plain", lq_off, 8))
        if lc and m >= n and n >= 64:
            out.append(("mixed", lq_off, 0))
    return out


def _jobs(device, chil, chim, chir, d, njobs, seed):
    import torch
    from .circuits import haar_random_matrix
    rng = np.random.default_rng(seed)

    def sites(n, a, b, scale):
        t = rng.normal(size=(n, a, d, b)) + 1j * rng.normal(size=(n, a, d, b))
        return torch.from_numpy((t * scale).astype(np.complex64)).to(device)
    m, n = chil * d, chir * d
    k = min(m, n)
    A, B = sites(njobs, chil, chim, 1.0 / max(chim, 1)), sites(njobs, chim, chir, 1.0)
    G = torch.from_numpy(np.stack([haar_random_matrix(2, d, seed + q) for q in range(njobs)])
                         .astype(np.complex64)).to(device)
    Ao = torch.empty((njobs, chil, d, k), dtype=torch.complex64, device=device)
    Bo = torch.empty((njobs, k, d, chir), dtype=torch.complex64, device=device)
    S = torch.zeros((njobs, k), dtype=torch.float32, device=device)
    table = np.zeros(njobs, dtype=_native.JOB_DTYPE)
    for q in range(njobs):
        r = table[q]
        r["a"], r["b"], r["gate"] = A[q].data_ptr(), B[q].data_ptr(), G[q].data_ptr()
        r["a_out"], r["b_out"], r["svals"] = Ao[q].data_ptr(), Bo[q].data_ptr(), S[q].data_ptr()
        r["chi_l"], r["chi_m"], r["chi_r"], r["k"], r["keep_left_canonical"] = chil, chim, chir, k, 1
    jobs = torch.from_numpy(table.view(np.uint8)).to(device)
    return (A, B, G, Ao, Bo, jobs), S


def _time(lib, keep, S, njobs, m, n, d, cand, reps, ws):
    import torch
    prec, lq_off, block = cand
    p = _native.SvdParams()
    p.precision = _native.PRECISION_MIXED if prec == "mixed" else _native.PRECISION_PLAIN
    p.lq_off, p.block_request = lq_off, block
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    jobs = keep[-1]
    times = []
    for r in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = lib.mps_apply_2q_batch(stream, ctypes.c_void_p(jobs.data_ptr()), njobs, m, n, d,
                                    ctypes.c_void_p(ws.data_ptr()), ws.numel(), ctypes.byref(p))
        e1.record()
        torch.cuda.synchronize()
        if rc != _native.MPS_OK:
            return None, None
        if r:
            times.append(e0.elapsed_time(e1))
    return float(np.median(times)), S.cpu().numpy().copy()


def tune(shapes, njobs_list=TUNE_BATCHES, reps: int = 3, device=None, log=print) -> Dict:
    """Times every candidate for each (chi_l, chi_m, chi_r, d) shape and batch
    size; returns {key: {settings..., "ms": {candidate: ms}}}."""
    import torch
    lib = _native.load()
    device = device or torch.device("cuda", torch.cuda.current_device())
    out = {}
    for (chil, chim, chir, d) in shapes:
        m, n = chil * d, chir * d
        for nj in njobs_list:
            keep, S = _jobs(device, chil, chim, chir, d, nj, 1000 + chil)
            ws = torch.empty(lib.mps_2q_workspace_bytes_mixed(nj, m, n, d), dtype=torch.uint8,
                             device=device)
            ref_ms, ref = _time(lib, keep, S, nj, m, n, d, ("plain", 0, 0), reps, ws)
            best, best_ms, res = ("plain", 0, 0), ref_ms, {}
            for cand in candidates(m, n):
                ms, sv = (ref_ms, ref) if cand == ("plain", 0, 0) else \
                    _time(lib, keep, S, nj, m, n, d, cand, reps, ws)
                if ms is None:
                    continue
                ok = np.all(np.abs(sv - ref) <= 1e-4 * ref[:, :1] + 1e-30)
                res["/".join(map(str, cand))] = round(ms, 4) if ok else None
                if ok and ms < best_ms:
                    best, best_ms = cand, ms
            k = key(m, n, d, nj)
            out[k] = {"precision": best[0], "lq_off": best[1], "block_request": best[2],
                      "ms": res, "shape": [chil, chim, chir, d], "njobs": nj}
            log(f"{k}: best {best} {best_ms:.3f} ms  {res}")
            del keep, ws
            torch.cuda.empty_cache()
    return out


WORKLOAD_SHAPES = [
    (32, 32, 32, 2), (64, 64, 64, 2), (128, 128, 128, 2), (256, 256, 256, 2),   # theta 64..512
    (64, 64, 64, 3), (192, 192, 192, 3),                                       # theta 192, 576
]


def main(argv=None):
    import argparse
    import platform
    import torch
    ap = argparse.ArgumentParser(description="tune the two-qudit call on this GPU")
    ap.add_argument("--out", default=TABLE_PATH)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    import __graft_entry__ as ge   # noqa: F401  (the library must be built)
    ge.build()
    t0 = time.time()
    entries = tune(WORKLOAD_SHAPES, reps=a.reps)
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump({"device": torch.cuda.get_device_name(0), "host": platform.machine(),
                   "seconds": round(time.time() - t0, 1), "entries": entries}, f, indent=1)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
