"""mps_cgemm_tc (tcgen05 tensor cores, bf16 three-piece split) through the C ABI.

Each case is compared with the same product in complex128 NumPy.  Tolerance:
every element within 1e-7 (1 + sqrt(k)) x (|row of opA| |column of opB|), the
bound an FP32 SIMT GEMM meets (the split keeps 2^-26 of each operand and the
six piece products drop terms below 2^-26 |a||b|; FP32 accumulation of the 2k
real terms adds ~sqrt(2k) 2^-24).  Plain TF32 or bf16 products miss it by two
to four orders of magnitude.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _cgemm(lib, fn, m, n, k, a, sam, sak, conj_a, b, sbk, sbn, conj_b, c, scm, scn, batch=0,
           bsa=0, bsb=0, bsc=0):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = getattr(lib, fn)(stream, m, n, k, ctypes.c_void_p(a.data_ptr()), sam, sak, conj_a,
                          ctypes.c_void_p(b.data_ptr()), sbk, sbn, conj_b,
                          ctypes.c_void_p(c.data_ptr()), scm, scn, batch, bsa, bsb, bsc)
    assert rc == 0, lib.mps_last_error()


def _rand(rng, *shape, scale=1.0):
    return ((rng.normal(size=shape) + 1j * rng.normal(size=shape)) * scale).astype(np.complex64)


def _bound(opa, opb):
    ra = np.linalg.norm(opa.astype(np.complex128), axis=1)
    cb = np.linalg.norm(opb.astype(np.complex128), axis=0)
    return np.outer(ra, cb)


def _tol(k):
    return 1e-7 * (1.0 + np.sqrt(k))


@pytest.mark.parametrize("m,n,k", [(128, 64, 32), (200, 100, 77), (512, 512, 256), (1, 3, 5),
                                   (576, 192, 576), (64, 700, 1000)])
def test_tc_gemm_matches_complex128(built_lib, cuda, m, n, k):
    rng = np.random.default_rng(m * 7919 + n * 31 + k)
    a = _rand(rng, m, k)
    b = _rand(rng, k, n, scale=1e-3)           # mixed magnitudes between operands
    ta, tb = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    tc_ = torch.full((m, n), float("nan"), dtype=torch.complex64, device=cuda)
    _cgemm(built_lib, "mps_cgemm_tc", m, n, k, ta, k, 1, 0, tb, n, 1, 0, tc_, n, 1)
    torch.cuda.synchronize()
    got = tc_.cpu().numpy().astype(np.complex128)
    ref = a.astype(np.complex128) @ b.astype(np.complex128)
    err = np.abs(got - ref)
    assert np.all(np.isfinite(got))
    assert np.all(err <= _tol(k) * _bound(a, b) + 1e-30), float(np.max(err / _bound(a, b)))
    flag = ctypes.c_int(-1)
    assert built_lib.mps_tc_error(ctypes.byref(flag)) == 0 and flag.value == 0


def test_tc_gemm_strides_conj_and_batch(built_lib, cuda):
    """opA = conj(A^T) read column-major, opB = conj(B) row-major, a strided
    output and three batch entries: every stride path of the fill."""
    rng = np.random.default_rng(3)
    m, n, k, nb = 150, 90, 130, 3
    A = _rand(rng, nb, k, m)                    # opA(i, t) = conj(A[z, t, i])
    B = _rand(rng, nb, k, n)
    ta, tb = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    out = torch.zeros((nb, n, m), dtype=torch.complex64, device=cuda)   # C^T storage
    _cgemm(built_lib, "mps_cgemm_tc", m, n, k, ta, 1, m, 1, tb, n, 1, 1, out, 1, m,
           batch=nb, bsa=k * m, bsb=k * n, bsc=n * m)
    torch.cuda.synchronize()
    got = out.cpu().numpy().transpose(0, 2, 1)
    for z in range(nb):
        opa = np.conj(A[z].T).astype(np.complex128)
        opb = np.conj(B[z]).astype(np.complex128)
        ref = opa @ opb
        assert np.all(np.abs(got[z] - ref) <= _tol(k) * _bound(opa, opb))


def test_tc_gemm_agrees_with_simt_gemm(built_lib, cuda):
    """The tensor-core product and the FP32 SIMT product of mps_cgemm agree to
    FP32 rounding on a chi=256 environment-sized product."""
    rng = np.random.default_rng(11)
    m = n = 256
    k = 512
    a, b = _rand(rng, m, k), _rand(rng, k, n)
    ta, tb = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    c1 = torch.zeros((m, n), dtype=torch.complex64, device=cuda)
    c2 = torch.zeros_like(c1)
    _cgemm(built_lib, "mps_cgemm_tc", m, n, k, ta, k, 1, 0, tb, n, 1, 0, c1, n, 1)
    _cgemm(built_lib, "mps_cgemm", m, n, k, ta, k, 1, 0, tb, n, 1, 0, c2, n, 1)
    torch.cuda.synchronize()
    d = np.abs(c1.cpu().numpy() - c2.cpu().numpy())
    assert np.max(d / _bound(a, b)) < 2 * _tol(k)
