"""mps_apply_2q_batch through the C ABI against NumPy/LAPACK (complex128).

Each job merges random sites with a Haar gate; the kernel's singular values,
truncated two-site block, isometry of the canonical factor and discarded
weight are compared with an SVD of the same merged matrix in complex128.
Tolerances (complex64 arithmetic): singular values |s - s_ref| <=
2e-5 s_ref + 2e-6 s_ref[0]; isometry to 2e-5; truncated block to
max(2e-5, 3x the error of LAPACK's complex64 SVD on the same input).
"""
import ctypes

import numpy as np
import pytest
import torch

from mpsim_gb300 import _native
from mpsim_gb300 import circuits as C

pytestmark = pytest.mark.gpu


def theta_of(a, b, g, d):
    chil, _, chim = a.shape
    chir = b.shape[2]
    m = (a.reshape(chil * d, chim) @ b.reshape(chim, d * chir)).reshape(chil, d, d, chir)
    th = np.einsum("xyab,labr->lxyr", g.reshape((d,) * 4), m)
    return th.reshape(chil * d, d * chir)


def make_job_inputs(rng, chil, chim, chir, d, rank=None, scale=1.0):
    a = (rng.normal(size=(chil, d, chim)) + 1j * rng.normal(size=(chil, d, chim))) * scale
    b = rng.normal(size=(chim, d, chir)) + 1j * rng.normal(size=(chim, d, chir))
    if rank is not None and chim > 0:
        a[..., rank:] = 0
    g = C.haar_random_matrix(2, d, int(rng.integers(1 << 30)))
    return a.astype(np.complex64), b.astype(np.complex64), g.astype(np.complex64)


def run_batch(lib, dev, specs, params=None):
    """specs: list of (a, b, g, k, lc).  Returns per-job dict of outputs."""
    d = specs[0][0].shape[1]
    njobs = len(specs)
    table = np.zeros(njobs, dtype=_native.JOB_DTYPE)
    keep = []
    outs = []
    max_m = max_n = 1
    for q, (a, b, g, k, lc) in enumerate(specs):
        chil, _, chim = a.shape
        chir = b.shape[2]
        ta = torch.from_numpy(a).to(dev)
        tb = torch.from_numpy(b).to(dev)
        tg = torch.from_numpy(np.ascontiguousarray(g)).to(dev)
        ao = torch.full((chil, d, k), float("nan"), dtype=torch.complex64, device=dev)
        bo = torch.full((k, d, chir), float("nan"), dtype=torch.complex64, device=dev)
        r = min(chil * d, chir * d)
        sv = torch.zeros(max(r, 1), dtype=torch.float32, device=dev)
        dc = torch.zeros(1, dtype=torch.float64, device=dev)
        st = torch.full((1,), -1, dtype=torch.int32, device=dev)
        keep += [ta, tb, tg]
        outs.append((ao, bo, sv, dc, st, r))
        row = table[q]
        row["a"], row["b"], row["gate"] = ta.data_ptr(), tb.data_ptr(), tg.data_ptr()
        row["a_out"] = ao.data_ptr() if ao.numel() else 0
        row["b_out"] = bo.data_ptr() if bo.numel() else 0
        row["svals"], row["discarded"], row["status"] = sv.data_ptr(), dc.data_ptr(), st.data_ptr()
        row["chi_l"], row["chi_m"], row["chi_r"], row["k"] = chil, chim, chir, k
        row["keep_left_canonical"] = int(lc)
        max_m, max_n = max(max_m, chil * d), max(max_n, chir * d)
    jobs = torch.from_numpy(table.view(np.uint8)).to(dev)
    p = params or _native.SvdParams()
    size_fn = (lib.mps_2q_workspace_bytes_mixed if p.precision == _native.PRECISION_MIXED
               else lib.mps_2q_workspace_bytes)
    nbytes = size_fn(njobs, max_m, max_n, d)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.mps_apply_2q_batch(stream, ctypes.c_void_p(jobs.data_ptr()), njobs, max_m, max_n, d,
                                ctypes.c_void_p(ws.data_ptr()), nbytes, ctypes.byref(p))
    torch.cuda.synchronize()
    res = []
    for ao, bo, sv, dc, st, r in outs:
        res.append(dict(a=ao.cpu().numpy(), b=bo.cpu().numpy(), s=sv.cpu().numpy()[:r],
                        disc=float(dc.cpu().numpy()[0]), status=int(st.cpu().numpy()[0])))
    return rc, res, p


def check_job(spec, out, d):
    a, b, g, k, lc = spec
    th = theta_of(a.astype(np.complex128), b.astype(np.complex128), g.astype(np.complex128), d)
    m, n = th.shape
    u, s, vh = np.linalg.svd(th, full_matrices=False)
    assert out["status"] == 0
    gs = out["s"].astype(np.float64)
    s0 = s[0] if s.size else 0.0
    assert np.all(np.abs(gs - s) <= 2e-5 * s + 2e-6 * s0 + 1e-30), np.max(np.abs(gs - s) / (s + s0))
    assert np.all(np.diff(gs) <= 0)
    assert np.isclose(out["disc"], float(np.sum(s[k:] ** 2)), rtol=1e-4, atol=1e-6 * s0 ** 2 + 1e-30)
    left = out["a"].reshape(m, k).astype(np.complex128)
    right = out["b"].reshape(k, n).astype(np.complex128)
    assert np.all(np.isfinite(left)) and np.all(np.isfinite(right))
    if k == 0:
        return
    best = (u[:, :k] * s[:k]) @ vh[:k]
    gap_ok = k == len(s) or s[k - 1] - s[k] > 1e-3 * s0
    if gap_ok:
        # Truncating at a spectral gap amplifies any complex64 SVD's rounding
        # by about s0/gap; the bar is 3x what LAPACK's complex64 SVD of the
        # same (complex64-rounded) theta achieves, and never below 2e-5.
        u4, s4, vh4 = np.linalg.svd(th.astype(np.complex64), full_matrices=False)
        lap = ((u4[:, :k] * s4[:k]) @ vh4[:k]).astype(np.complex128)
        nb = max(np.linalg.norm(best), 1e-30)
        lap_err = np.linalg.norm(lap - best) / nb
        err = np.linalg.norm(left @ right - best) / nb
        assert err < max(2e-5, 3 * lap_err), (err, lap_err)
    iso = left if lc else right.T
    gram = iso.conj().T @ iso if lc else right @ right.conj().T
    assert np.allclose(gram, np.eye(k), atol=2e-5), np.max(np.abs(gram - np.eye(k)))


CASES = [
    # chil, chim, chir, d, rank, k(None=all), lc
    (1, 1, 1, 2, None, None, True),
    (1, 1, 4, 2, None, None, True),          # wide 2 x 8
    (4, 1, 1, 2, None, None, False),         # tall 8 x 2
    (8, 2, 8, 2, None, None, True),          # rank 8 < 16: zero singular values kept
    (8, 2, 8, 2, None, None, False),
    (8, 2, 8, 2, None, 12, True),
    (32, 16, 8, 2, None, 10, True),          # tall 64 x 16
    (16, 64, 64, 2, None, 20, False),        # wide 32 x 128
    (16, 64, 64, 2, None, 20, True),
    (21, 30, 17, 3, None, 40, True),         # qutrits, ragged sizes
    (64, 64, 64, 3, None, 96, False),        # 192 x 192
    (4, 0, 4, 2, None, 8, True),             # zero middle bond: theta = 0
    (4, 0, 4, 2, None, 8, False),
    (6, 5, 6, 2, 1, 7, True),                # rank-1 A: exact zero directions
    (12, 12, 12, 2, None, 0, True),          # keep nothing
]


@pytest.mark.parametrize("case", CASES)
def test_single_job(built_lib, cuda, case):
    chil, chim, chir, d, rank, k, lc = case
    rng = np.random.default_rng(abs(hash(case)) % (1 << 31))
    a, b, g = make_job_inputs(rng, chil, chim, chir, d, rank)
    r = min(chil * d, chir * d)
    k = r if k is None else min(k, r)
    rc, res, _ = run_batch(built_lib, cuda, [(a, b, g, k, lc)])
    assert rc == 0, _native.last_error()
    check_job((a, b, g, k, lc), res[0], d)


@pytest.mark.parametrize("chi,d,k", [(256, 2, 256), (192, 3, 192), (128, 2, 128)])
def test_full_size_job(built_lib, cuda, chi, d, k):
    """theta of 512x512 / 576x576 / 256x256, the workloads' largest."""
    rng = np.random.default_rng(chi * 10 + d)
    a, b, g = make_job_inputs(rng, chi, chi, chi, d, scale=1.0 / chi)
    for lc in (True, False):
        rc, res, p = run_batch(built_lib, cuda, [(a, b, g, k, lc)])
        assert rc == 0, _native.last_error()
        check_job((a, b, g, k, lc), res[0], d)
        assert p.sweeps_out < 40


def test_lq_preconditioned_mixed_batch(built_lib, cuda):
    """Tall and square left-canonical jobs of 64 to 768 columns are solved on
    the L factor of theta (theta = L Q, blocked Householder from the right);
    a batch mixing them with wide, right-canonical and narrow jobs, a ragged
    last panel (90 columns) and tall jobs (rows below the last panel) must
    match LAPACK like every other job."""
    rng = np.random.default_rng(23)
    shapes = [  # chil, chim, chir, k, lc  (d = 2)
        (128, 96, 128, 200, True),      # 256 x 256
        (100, 60, 45, 70, True),        # tall 200 x 90: last panel 26 rows
        (192, 64, 64, 100, True),       # tall 384 x 128
        (96, 64, 96, 150, False),       # right-canonical: not factorised
        (16, 32, 64, 20, True),         # wide 32 x 128: not factorised
        (16, 8, 16, 32, True),          # 32 x 32: below the size threshold
    ]
    specs = []
    for chil, chim, chir, k, lc in shapes:
        a, b, g = make_job_inputs(rng, chil, chim, chir, 2, scale=1.0 / chim)
        specs.append((a, b, g, k, lc))
    rc, res, p = run_batch(built_lib, cuda, specs)
    assert rc == 0, _native.last_error()
    for spec, out in zip(specs, res):
        check_job(spec, out, 2)


@pytest.mark.parametrize("lc", [True, False])
def test_graded_spectrum_keeps_isometry(built_lib, cuda, lc):
    """Singular values spread over twelve decades, all kept.  Pairs of
    columns below ~1e-10 in norm have |gamma|^2 below FP32's normal range
    (the L factor's columns are graded like this from the first sweep); the
    rotation test and angles must still see them, or the kept factor loses
    its isometry in those directions."""
    rng = np.random.default_rng(31)
    a, b, g = make_job_inputs(rng, 128, 128, 128, 2, scale=1.0 / 128)
    a = (a * (10.0 ** (-12.0 * np.arange(128) / 127))).astype(np.complex64)
    rc, res, _ = run_batch(built_lib, cuda, [(a, b, g, 256, lc)])
    assert rc == 0, _native.last_error()
    check_job((a, b, g, 256, lc), res[0], 2)


@pytest.mark.parametrize("chi", [384, 400])
def test_lq_size_limit(built_lib, cuda, chi):
    """768 columns is the widest factorised job (its 32-row panel fills the
    shared memory); 800 columns is solved on theta itself."""
    rng = np.random.default_rng(chi)
    a, b, g = make_job_inputs(rng, chi, chi // 2, chi, 2, scale=1.0 / chi)
    rc, res, p = run_batch(built_lib, cuda, [(a, b, g, chi, True)])
    assert rc == 0, _native.last_error()
    check_job((a, b, g, chi, True), res[0], 2)
    assert p.sweeps_out < 40


@pytest.mark.parametrize("scale", [1e-20, 1e-9, 1e15])
def test_scale_invariance(built_lib, cuda, scale):
    """theta scaled far from 1: squared norms of 1e-40 are below FP32's
    normal range unless the kernel rescales theta (exactly, by a power of
    two) before the SVD; the same relative tolerances must hold."""
    rng = np.random.default_rng(17)
    for lc in (True, False):
        a, b, g = make_job_inputs(rng, 64, 64, 64, 2, scale=scale / 64)
        rc, res, _ = run_batch(built_lib, cuda, [(a, b, g, 100, lc)])
        assert rc == 0, _native.last_error()
        check_job((a, b, g, 100, lc), res[0], 2)


def test_batch_equals_single(built_lib, cuda):
    rng = np.random.default_rng(7)
    specs = []
    for (chil, chim, chir, k, lc) in [(32, 16, 64, 40, True), (8, 4, 8, 16, False), (64, 64, 64, 100, True),
                                      (1, 1, 2, 2, True), (40, 33, 2, 4, False)]:
        a, b, g = make_job_inputs(rng, chil, chim, chir, 2)
        specs.append((a, b, g, min(k, min(chil, chir) * 2), lc))
    rc, res, _ = run_batch(built_lib, cuda, specs)
    assert rc == 0, _native.last_error()
    for spec, out in zip(specs, res):
        check_job(spec, out, 2)
        rc1, one, _ = run_batch(built_lib, cuda, [spec])
        assert rc1 == 0
        assert np.allclose(one[0]["s"], out["s"], rtol=1e-6, atol=1e-7 * max(out["s"][0], 1e-30))


def test_nonfinite_input_reports(built_lib, cuda):
    rng = np.random.default_rng(9)
    a, b, g = make_job_inputs(rng, 8, 8, 8, 2)
    a[0, 0, 0] = np.nan
    rc, res, _ = run_batch(built_lib, cuda, [(a, b, g, 8, True)])
    assert rc == _native.MPS_ERR_NONFINITE
    assert res[0]["status"] & _native.STATUS_NONFINITE


def test_sweep_cap_reports(built_lib, cuda):
    rng = np.random.default_rng(10)
    a, b, g = make_job_inputs(rng, 64, 64, 64, 2)
    p = _native.SvdParams(1, 0.0, 0, 0)
    rc, res, p = run_batch(built_lib, cuda, [(a, b, g, 64, True)], params=p)
    assert rc == _native.MPS_ERR_NOT_CONVERGED
    assert res[0]["status"] & _native.STATUS_NOT_CONVERGED
    assert p.sweeps_out == 1


def test_wait_timeout_reports_and_recovers(built_lib, cuda):
    """The sweep kernel's round-dependency waits are bounded: the stall test
    hook makes one wait target a round that never completes; with a small
    wait limit the call must return MPS_ERR_TIMEOUT (no hang, no fault), and
    the next call on the same context must work."""
    rng = np.random.default_rng(12)
    a, b, g = make_job_inputs(rng, 64, 64, 64, 2)          # 128 columns: 7 rounds per sweep
    p = _native.SvdParams(0, 0.0, 0, 0, 2000, 1)
    rc, _, _ = run_batch(built_lib, cuda, [(a, b, g, 64, True)], params=p)
    assert rc == _native.MPS_ERR_TIMEOUT
    assert "expired" in _native.last_error()
    rc, res, _ = run_batch(built_lib, cuda, [(a, b, g, 64, True)])
    assert rc == 0, _native.last_error()
    check_job((a, b, g, 64, True), res[0], 2)
