"""The allocation-free entry point, mps_apply_2q_batch_noalloc.

It serves callers that cannot allocate device memory themselves -- e.g. an
application whose own pool owns the GPU's memory, or a plugin host that gives
its plugins no allocator -- by taking its scratch from a fixed static device
array instead of a caller workspace.  This test calls it through the C ABI
twice in a row (the second call runs on the scratch the first one left
behind) and checks both results against mps_apply_2q_batch with a workspace,
within the tolerances of test_gpu_svd_kernel: singular values to
2e-5 s + 2e-6 s_0, the truncated two-site block to 2e-5 relative.  It also
checks that jobs needing more scratch than the array holds are refused with
MPS_ERR_WORKSPACE.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

from mpsim_gb300 import _native
from mpsim_gb300 import circuits as C

pytestmark = pytest.mark.gpu


def _jobs(dev, specs):
    d = specs[0][0].shape[1]
    table = np.zeros(len(specs), dtype=_native.JOB_DTYPE)
    keep, outs = [], []
    max_m = max_n = 1
    for q, (a, b, g, k, lc) in enumerate(specs):
        chil, _, chim = a.shape
        chir = b.shape[2]
        ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        tg = torch.from_numpy(np.ascontiguousarray(g)).to(dev)
        ao = torch.full((chil, d, k), float("nan"), dtype=torch.complex64, device=dev)
        bo = torch.full((k, d, chir), float("nan"), dtype=torch.complex64, device=dev)
        r = min(chil, chir) * d
        sv = torch.zeros(r, dtype=torch.float32, device=dev)
        st = torch.full((1,), -1, dtype=torch.int32, device=dev)
        keep += [ta, tb, tg]
        outs.append((ao, bo, sv, st))
        row = table[q]
        row["a"], row["b"], row["gate"] = ta.data_ptr(), tb.data_ptr(), tg.data_ptr()
        row["a_out"], row["b_out"] = ao.data_ptr(), bo.data_ptr()
        row["svals"], row["status"] = sv.data_ptr(), st.data_ptr()
        row["chi_l"], row["chi_m"], row["chi_r"], row["k"] = chil, chim, chir, k
        row["keep_left_canonical"] = int(lc)
        max_m, max_n = max(max_m, chil * d), max(max_n, chir * d)
    jobs = torch.from_numpy(table.view(np.uint8)).to(dev)
    return jobs, keep, outs, max_m, max_n, d


def _results(outs):
    torch.cuda.synchronize()
    return [(a.cpu().numpy(), b.cpu().numpy(), s.cpu().numpy(), int(st.cpu().numpy()[0]))
            for a, b, s, st in outs]


def _specs(seed):
    rng = np.random.default_rng(seed)
    specs = []
    for chil, chim, chir, k, lc in [(128, 128, 128, 128, True), (64, 32, 96, 50, False),
                                    (8, 2, 8, 16, True), (33, 20, 7, 9, True)]:
        a = (rng.normal(size=(chil, 2, chim)) + 1j * rng.normal(size=(chil, 2, chim))) / chil
        b = rng.normal(size=(chim, 2, chir)) + 1j * rng.normal(size=(chim, 2, chir))
        g = C.haar_random_matrix(2, 2, int(rng.integers(1 << 30)))
        specs.append((a.astype(np.complex64), b.astype(np.complex64), g.astype(np.complex64),
                      min(k, 2 * min(chil, chir)), lc))
    return specs


def _run_workspace(lib, dev, specs):
    jobs, keep, outs, mm, mn, d = _jobs(dev, specs)
    nbytes = lib.mps_2q_workspace_bytes(len(specs), mm, mn, d)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.mps_apply_2q_batch(stream, ctypes.c_void_p(jobs.data_ptr()), len(specs), mm, mn, d,
                                ctypes.c_void_p(ws.data_ptr()), nbytes,
                                ctypes.byref(_native.SvdParams()))
    assert rc == 0, _native.last_error()
    return _results(outs)


def _run_noalloc(lib, dev, specs):
    jobs, keep, outs, mm, mn, d = _jobs(dev, specs)
    assert lib.mps_2q_workspace_bytes(len(specs), mm, mn, d) <= _native.NOALLOC_SCRATCH_BYTES
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.mps_apply_2q_batch_noalloc(stream, ctypes.c_void_p(jobs.data_ptr()), len(specs),
                                        mm, mn, d, ctypes.byref(_native.SvdParams()))
    assert rc == 0, _native.last_error()
    return _results(outs)


def _close(ref, got):
    for (ra, rb, rs, rst), (ga, gb, gs, gst) in zip(ref, got):
        assert rst == 0 and gst == 0
        s0 = rs[0]
        assert np.all(np.abs(gs - rs) <= 2e-5 * rs + 2e-6 * s0)
        k = ra.shape[2]
        m, n = ra.shape[0] * ra.shape[1], rb.shape[1] * rb.shape[2]
        pr = ra.reshape(m, k).astype(np.complex128) @ rb.reshape(k, n).astype(np.complex128)
        pg = ga.reshape(m, k).astype(np.complex128) @ gb.reshape(k, n).astype(np.complex128)
        assert np.linalg.norm(pg - pr) <= 2e-5 * np.linalg.norm(pr)


def test_noalloc_matches_workspace_entry_point_twice(built_lib, cuda):
    specs = _specs(11)
    ref = _run_workspace(built_lib, cuda, specs)
    first = _run_noalloc(built_lib, cuda, specs)
    _close(ref, first)
    second = _run_noalloc(built_lib, cuda, _specs(11))
    _close(ref, second)


def test_noalloc_rejects_oversized_jobs(built_lib, cuda):
    rng = np.random.default_rng(3)
    big = []
    for _ in range(8):                      # eight theta 512x512 jobs need > 32 MiB
        a = (rng.normal(size=(256, 2, 256)) + 0j).astype(np.complex64)
        b = (rng.normal(size=(256, 2, 256)) + 0j).astype(np.complex64)
        big.append((a, b, np.eye(4, dtype=np.complex64), 256, True))
    jobs, keep, outs, mm, mn, d = _jobs(cuda, big)
    assert built_lib.mps_2q_workspace_bytes(8, mm, mn, d) > _native.NOALLOC_SCRATCH_BYTES
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = built_lib.mps_apply_2q_batch_noalloc(stream, ctypes.c_void_p(jobs.data_ptr()), 8, mm, mn,
                                              d, ctypes.byref(_native.SvdParams()))
    assert rc == _native.MPS_ERR_WORKSPACE
    assert "scratch" in _native.last_error()
