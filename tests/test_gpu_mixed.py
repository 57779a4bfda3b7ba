"""The mixed-precision form (MPS_PRECISION_MIXED: tensor-core block Jacobi
sweeps with split-bf16 tcgen05 Gram and rotation GEMMs) against complex128
LAPACK and against the reference's own complex128 run.

Per job the checks are the plain path's (tests/test_gpu_svd_kernel.py
check_job: singular values within 2e-5 s + 2e-6 s_0, isometry to 2e-5, the
truncated block within max(2e-5, 3x LAPACK complex64's error), discarded
weight to 1e-4 relative) plus the figures the precision form reports against
the FP64 oracle: the two-site block's infidelity after truncation (<= 1e-5),
the largest singular-value relative error over the kept values (<= 1e-5 for
values above 1e-3 s_0) and the truncation-weight error (<= 1e-4 relative).
"""
import os

import numpy as np
import pytest
import torch

from mpsim_gb300 import _native
from test_gpu_svd_kernel import check_job, make_job_inputs, run_batch, theta_of

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def mixed_params(**kw):
    p = _native.SvdParams()
    p.precision = _native.PRECISION_MIXED
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def precision_report(spec, out, d):
    """(block infidelity, max kept sv relative error, truncation-weight
    relative error) of one job against complex128 LAPACK."""
    a, b, g, k, lc = spec
    th = theta_of(a.astype(np.complex128), b.astype(np.complex128), g.astype(np.complex128), d)
    m, n = th.shape
    u, s, vh = np.linalg.svd(th, full_matrices=False)
    best = (u[:, :k] * s[:k]) @ vh[:k]
    got = out["a"].reshape(m, k).astype(np.complex128) @ out["b"].reshape(k, n).astype(np.complex128)
    ov = abs(np.vdot(best, got)) ** 2 / (np.vdot(best, best).real * np.vdot(got, got).real)
    keep = s[:k] > 1e-3 * s[0]
    sv_err = float(np.max(np.abs(out["s"][:k][keep] - s[:k][keep]) / s[:k][keep]))
    w = float(np.sum(s[k:] ** 2))
    w_err = abs(out["disc"] - w) / max(w, 1e-30)
    return 1.0 - ov, sv_err, w_err


@pytest.mark.parametrize("chi,d,k", [(256, 2, 256), (192, 3, 192), (128, 2, 128), (32, 2, 64)])
def test_mixed_full_size_job(built_lib, cuda, chi, d, k):
    """theta of 512x512 / 576x576 / 256x256 / 64x64: the workloads' shapes."""
    rng = np.random.default_rng(chi * 10 + d + 1)
    a, b, g = make_job_inputs(rng, chi, chi, chi, d, scale=1.0 / chi)
    k = min(k, chi * d)
    rc, res, p = run_batch(built_lib, cuda, [(a, b, g, k, True)], params=mixed_params())
    assert rc == 0, _native.last_error()
    assert p.block_cols == 32
    check_job((a, b, g, k, True), res[0], d)
    infid, sv_err, w_err = precision_report((a, b, g, k, True), res[0], d)
    assert infid <= 1e-5 and sv_err <= 1e-5 and w_err <= 1e-4, (infid, sv_err, w_err)
    assert p.sweeps_out < 40


def test_mixed_matches_plain_per_gate(built_lib, cuda):
    """The same eight chi=256 gates through both forms: singular values agree
    to the plain form's own accuracy."""
    rng = np.random.default_rng(5)
    specs = []
    for _ in range(8):
        a, b, g = make_job_inputs(rng, 256, 256, 256, 2, scale=1.0 / 256)
        specs.append((a, b, g, 256, True))
    rc, mix, _ = run_batch(built_lib, cuda, specs, params=mixed_params())
    assert rc == 0, _native.last_error()
    rc, pln, _ = run_batch(built_lib, cuda, specs)
    assert rc == 0, _native.last_error()
    for spec, om, op in zip(specs, mix, pln):
        check_job(spec, om, 2)
        s0 = op["s"][0]
        assert np.all(np.abs(om["s"] - op["s"]) <= 4e-5 * op["s"] + 4e-6 * s0)


def test_mixed_batch_of_shapes(built_lib, cuda):
    """Tall left-canonical jobs of 64 to 576 columns in one call, ragged
    block counts (90 columns: a zero-padded last block), rows below the LQ
    panels."""
    rng = np.random.default_rng(41)
    shapes = [(128, 96, 128, 200), (100, 60, 45, 70), (192, 64, 64, 100), (32, 20, 32, 64),
              (96, 96, 48, 96)]
    specs = []
    for chil, chim, chir, k in shapes:
        a, b, g = make_job_inputs(rng, chil, chim, chir, 2, scale=1.0 / chim)
        specs.append((a, b, g, k, True))
    rc, res, _ = run_batch(built_lib, cuda, specs, params=mixed_params())
    assert rc == 0, _native.last_error()
    for spec, out in zip(specs, res):
        check_job(spec, out, 2)


def test_mixed_graded_spectrum(built_lib, cuda):
    """Twelve decades of singular values, all kept: the Gram-based rotations
    must still orthogonalise the small columns."""
    rng = np.random.default_rng(31)
    a, b, g = make_job_inputs(rng, 128, 128, 128, 2, scale=1.0 / 128)
    a = (a * (10.0 ** (-12.0 * np.arange(128) / 127))).astype(np.complex64)
    rc, res, _ = run_batch(built_lib, cuda, [(a, b, g, 256, True)], params=mixed_params())
    assert rc == 0, _native.last_error()
    check_job((a, b, g, 256, True), res[0], 2)


@pytest.mark.parametrize("scale", [1e-20, 1e15])
def test_mixed_scale_invariance(built_lib, cuda, scale):
    rng = np.random.default_rng(17)
    a, b, g = make_job_inputs(rng, 64, 64, 64, 2, scale=scale / 64)
    rc, res, _ = run_batch(built_lib, cuda, [(a, b, g, 100, True)], params=mixed_params())
    assert rc == 0, _native.last_error()
    check_job((a, b, g, 100, True), res[0], 2)


def test_mixed_call_runs_other_jobs_in_the_plain_sweeps(built_lib, cuda):
    """One mixed call with tensor-core jobs (left-canonical, tall, 64+
    columns) and jobs of every other kind: right-canonical (they need the
    accumulated V), wide, and of fewer than 64 columns.  The others take the
    SIMT sweeps of the same call: each job passes the plain path's checks, and
    the other jobs' results equal a plain call's bit for bit."""
    rng = np.random.default_rng(3)
    specs = []
    for chil, chim, chir, d, k, lc in [(128, 64, 128, 2, 256, True),    # tensor-core
                                       (64, 64, 64, 2, 64, False),      # right-canonical
                                       (32, 64, 128, 2, 64, True),      # wide (m < n)
                                       (16, 16, 16, 2, 32, True),       # 32 columns
                                       (96, 96, 96, 2, 192, True)]:     # tensor-core
        a, b, g = make_job_inputs(rng, chil, chim, chir, d, scale=1.0 / chim)
        specs.append((a, b, g, k, lc))
    rc, mix, p = run_batch(built_lib, cuda, specs, params=mixed_params())
    assert rc == 0, _native.last_error()
    assert p.block_cols == 32
    rc, pln, _ = run_batch(built_lib, cuda, specs)
    assert rc == 0, _native.last_error()
    for q, (spec, om, op) in enumerate(zip(specs, mix, pln)):
        check_job(spec, om, 2)
        if q in (1, 2, 3):
            for key in ("a", "b", "s"):
                assert np.array_equal(om[key], op[key]), (q, key)


def test_mixed_needs_its_workspace_size(built_lib, cuda):
    """A mixed call given only the plain form's workspace (no room for the
    piece planes) is refused before any launch."""
    import ctypes
    rng = np.random.default_rng(4)
    a, b, g = make_job_inputs(rng, 64, 64, 64, 2)
    small = built_lib.mps_2q_workspace_bytes(1, 128, 128, 2)
    assert built_lib.mps_2q_workspace_bytes_mixed(1, 128, 128, 2) > small
    ws = torch.empty(small, dtype=torch.uint8, device=cuda)
    jobs = torch.zeros(_native.JOB_DTYPE.itemsize, dtype=torch.uint8, device=cuda)
    p = mixed_params()
    rc = built_lib.mps_apply_2q_batch(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                                      ctypes.c_void_p(jobs.data_ptr()), 1, 128, 128, 2,
                                      ctypes.c_void_p(ws.data_ptr()), small, ctypes.byref(p))
    assert rc == _native.MPS_ERR_WORKSPACE


def test_mixed_circuit_10q_matches_reference_complex128(built_lib, cuda):
    """The 10-qubit depth-10 untruncated workload with precision="mixed"
    (its merged matrices are at most 32 x 32, so every gate takes the plain
    form): wavefunction infidelity against the reference's complex128 run
    below 1e-9 and amplitudes within 2e-6 of its complex64 run, exactly the
    plain form's bar."""
    from mpsim_gb300 import circuits as C
    from mpsim_gb300.core import MPS
    fx = np.load(os.path.join(GOLDEN, "brickwork_10q_d10_full.npz"))
    circ = C.workload("brickwork_10q_d10_full")
    mps = MPS(circ.nqudits, circ.d, precision="mixed")
    for lay in circ.layers:
        mps.apply_layer(lay.one_q, lay.pair_left, lay.two_q)
    got = mps.wavefunction().astype(np.complex128)
    ref = fx["ref_c128_wavefunction"]
    infid = 1.0 - abs(np.vdot(ref, got)) ** 2 / (np.vdot(ref, ref).real * np.vdot(got, got).real)
    assert infid < 1e-9, infid
    assert np.allclose(got, fx["ref_c64_wavefunction"], atol=2e-6)


@pytest.mark.parametrize("nq,depth,d", [(14, 10, 2), (9, 8, 3)])
def test_mixed_circuit_against_dense_fp64(built_lib, cuda, nq, depth, d):
    """Untruncated brickwork circuits whose middle gates reach 64 to 128
    columns (14 qubits; 9 qutrits) with precision="mixed", against the dense
    complex128 evolution of the same gates: wavefunction infidelity <= 1e-5
    (the precision form's target) and the plain form's result to 1e-6."""
    from mpsim_gb300 import circuits as C
    from mpsim_gb300.core import MPS
    from oracle.dense import DenseState
    circ = C.brickwork(nq, depth, d=d, maxsvals=None, seed=11)
    mix = MPS(nq, d, precision="mixed", record_svals=True)
    pln = MPS(nq, d)
    st = DenseState(nq, d)
    for lay in circ.layers:
        mix.apply_layer(lay.one_q, lay.pair_left, lay.two_q)
        pln.apply_layer(lay.one_q, lay.pair_left, lay.two_q)
        for i in range(nq):
            st.apply_one(lay.one_q[i], i)
        for p, i in enumerate(lay.pair_left):
            st.apply_two(lay.two_q[p], int(i), int(i) + 1)
    ref = st.vector()
    got = mix.wavefunction().astype(np.complex128)
    infid = 1.0 - abs(np.vdot(ref, got)) ** 2 / (np.vdot(ref, ref).real * np.vdot(got, got).real)
    assert infid <= 1e-5, infid
    assert np.max(np.abs(got - pln.wavefunction())) < 1e-6 * max(1.0, np.max(np.abs(got)))
    big = [h for h in mix.svals_history if len(h[0]) >= 64]
    assert big, "no gate reached the tensor-core sweeps"
