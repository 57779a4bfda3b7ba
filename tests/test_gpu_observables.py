"""Observables, splits and non-unitary gates on the GPU against the
reference's own outputs (tests/golden/observables.npz, written by
tests/golden/make_golden.py from the reference's mpsim/core.py).

Reduced density matrices and marginals go through mps_cgemm and
mps_site_marginals; from_wavefunction and the orthonormalisations through the
Jacobi kernel's given-matrix jobs.  Tolerances are complex64 (2e-6 absolute on
O(1) values, 5e-6 after a truncating circuit); seeded samples must be the
reference's exact draws.
"""
import importlib.util
import os

import numpy as np
import pytest

from mpsim_gb300 import MPS, MPSOperation
from mpsim_gb300 import circuits as C
from mpsim_gb300 import gates as G

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)
STATES = {s[0]: s[1:] for s in make_golden.OBS_STATES}
RDM = make_golden.OBS_RDM


@pytest.fixture(scope="module")
def z():
    return np.load(os.path.join(GOLDEN, "observables.npz"))


def gpu_state(name):
    n, d, depth, maxs, seed = STATES[name]
    circ = C.brickwork(n, depth, d=d, maxsvals=maxs, seed=seed)
    m = MPS(n, d)
    kw = {} if maxs is None else {"maxsvals": maxs}
    for kind, sites, mat in circ.operations():
        if kind == 1:
            m.apply_one_qudit_gate(np.asarray(mat), sites[0])
        else:
            m.apply_two_qudit_gate(np.asarray(mat).reshape((d,) * 4), sites[0], sites[1], **kw)
    return m


def tol(name):
    return 5e-6 if STATES[name][3] is not None else 2e-6


@pytest.mark.parametrize("name", list(STATES))
def test_rdm_and_marginals(cuda, z, name):
    m = gpu_state(name)
    assert np.allclose(m.wavefunction(), z[f"{name}_wf"], atol=tol(name))
    for idx in RDM[name]:
        key = "_".join(str(i) for i in idx)
        rho = m.reduced_density_matrix(list(idx))
        assert rho.shape == z[f"{name}_rdm_{key}"].shape
        assert np.allclose(rho, z[f"{name}_rdm_{key}"], atol=tol(name)), idx
    marg = m.site_marginals()
    assert marg.dtype == np.float32
    assert np.allclose(marg, z[f"{name}_marginals"], atol=tol(name))


def test_rdm_argument_errors(cuda):
    m = MPS(4)
    with pytest.raises(ValueError):
        m.reduced_density_matrix([1, 1])
    with pytest.raises(IndexError):
        m.reduced_density_matrix([0, 4])
    with pytest.raises(IndexError):
        m.reduced_density_matrix(-1)
    assert np.allclose(m.reduced_density_matrix(2), np.diag([1, 0]))


def test_samples_equal_reference_draws(cuda, z):
    q6 = gpu_state("q6")
    np.random.seed(7)
    assert np.array_equal(np.asarray(q6.sample(25)), z["q6_samples"])
    np.random.seed(8)
    hist = q6.sample(40, as_hist=True)
    assert sorted(hist) == list(z["q6_hist_keys"])
    assert [hist[k] for k in sorted(hist)] == list(z["q6_hist_counts"])
    np.random.seed(9)
    assert list(gpu_state("t4").sample(20, as_string=True)) == list(z["t4_samples"])
    with pytest.raises(ValueError):
        q6.sample(0)
    with pytest.raises(ValueError):
        q6.sample(2.0)
    # a truncated state's marginals do not sum to one: np.random.choice
    # refuses them, as it does in the reference
    with pytest.raises(ValueError):
        gpu_state("q8trunc").sample(1)


@pytest.mark.parametrize("name,n,d", [("fw_q6", 6, 2), ("fw_t4", 4, 3)])
def test_from_wavefunction(cuda, z, name, n, d):
    m = MPS.from_wavefunction(z[f"{name}_psi"], n, d)
    assert np.allclose(m.wavefunction(), z[f"{name}_wf"], atol=2e-6)
    assert list(m.bond_dimensions()) == list(z[f"{name}_bonds"])
    assert m.is_valid()


def test_from_wavefunction_errors_and_limit(cuda):
    with pytest.raises(TypeError):
        MPS.from_wavefunction("01", 2)
    with pytest.raises(ValueError):
        MPS.from_wavefunction(np.zeros((2, 2)), 2)
    with pytest.raises(ValueError):
        MPS.from_wavefunction(np.zeros(2), 1)
    with pytest.raises(ValueError):
        MPS.from_wavefunction(np.zeros(8), 2)
    # a product state: the zero singular values are kept, as split_node does
    psi = np.zeros(2 ** 5, np.complex64)
    psi[0b10110] = 1.0
    m = MPS.from_wavefunction(psi, 5)
    assert np.allclose(m.wavefunction(), psi, atol=1e-6)
    assert list(m.bond_dimensions()) == [2, 4, 4, 2]
    # the middle bond (2^11) reaches the Jacobi kernel's 1792 rows
    with pytest.raises(NotImplementedError):
        MPS.from_wavefunction(np.ones(2 ** 22) / 2048.0, 22)


@pytest.mark.parametrize("n,d,kind", [(14, 2, "haar"), (16, 2, "product"), (9, 3, "haar"),
                                      (13, 2, "ghz"), (21, 2, "haar"), (13, 3, "ghz")])
def test_from_wavefunction_long_splits(cuda, n, d, kind):
    """States whose splits are longer than the Jacobi kernel's 1792 rows (the
    column-block compression of _wide_left_svd): the state comes back, with
    the reference's bond dimensions min(d^i, d^(n-i)) (all values kept, as
    split_node does, zeros included)."""
    rng = np.random.default_rng(n * 10 + d)
    size = d ** n
    if kind == "haar":
        psi = (rng.normal(size=size) + 1j * rng.normal(size=size)).astype(np.complex64)
    elif kind == "product":
        psi = np.zeros(size, np.complex64)
        psi[int(rng.integers(size))] = 1.0
    else:
        psi = np.zeros(size, np.complex64)
        psi[0] = psi[-1] = 1.0
    psi /= np.linalg.norm(psi)
    m = MPS.from_wavefunction(psi, n, d)
    assert list(m.bond_dimensions()) == [min(d ** i, d ** (n - i)) for i in range(1, n)]
    wf = m.wavefunction().reshape(-1)
    a, b = psi.astype(np.complex128), wf.astype(np.complex128)
    fid = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
    assert fid > 1.0 - 1e-9
    assert np.max(np.abs(wf - psi)) < 4e-6
    assert m.is_valid()


def test_orthonormalize(cuda, z):
    m = gpu_state("q6")
    m.orthonormalize_right_edge_of(2)
    assert np.allclose(m.wavefunction(), z["ortho_r2_wf"], atol=2e-6)
    assert list(m.bond_dimensions()) == list(z["ortho_r2_bonds"])
    # site 2 is now an isometry over (left bond, digit)
    s2 = m.sites[2].reshape(-1, m.sites[2].shape[2]).cpu().numpy().astype(np.complex128)
    assert np.allclose(s2.conj().T @ s2, np.eye(s2.shape[1]), atol=2e-5)
    m.orthonormalize_left_edge_of(4)
    assert np.allclose(m.wavefunction(), z["ortho_l4_wf"], atol=2e-6)
    assert list(m.bond_dimensions()) == list(z["ortho_l4_bonds"])
    s4 = m.sites[4].reshape(m.sites[4].shape[0], -1).cpu().numpy().astype(np.complex128)
    assert np.allclose(s4 @ s4.conj().T, np.eye(s4.shape[0]), atol=2e-5)
    with pytest.raises(ValueError):
        m.orthonormalize_right_edge_of(5)
    with pytest.raises(ValueError):
        m.orthonormalize_left_edge_of(0)


def test_non_unitary_gates(cuda, z):
    m = MPS(4)
    m.h(0)
    for i in range(3):
        m.cnot(i, i + 1)
    m.apply_one_qudit_gate(G.computational_basis_projector(0), 1)
    assert np.allclose(m.wavefunction(), z["ghz_proj_wf"], atol=2e-6)
    assert list(m.bond_dimensions()) == list(z["ghz_proj_bonds"])
    damp = np.array([[1.0, 0.0], [0.0, 0.4]], dtype=np.complex64)
    for tag, kw in (("default", {}), ("noortho", {"ortho_after_non_unitary": False}),
                    ("norenorm", {"renormalize_after_non_unitary": False}), ("end", {})):
        m = gpu_state("q6")
        m.apply_one_qudit_gate(damp, 5 if tag == "end" else 3, **kw)
        assert np.allclose(m.wavefunction(), z[f"nonunit_{tag}_wf"], atol=2e-6), tag
        assert list(m.bond_dimensions()) == list(z[f"nonunit_{tag}_bonds"]), tag
        assert abs(m.norm() - float(z[f"nonunit_{tag}_norm"])) < 2e-6, tag


def test_expectation_values(cuda, z):
    m = gpu_state("q6")
    assert abs(m.expectation(MPSOperation(G.zgate(), 1)) - float(z["expect_z1"])) < 1e-5
    assert abs(m.expectation(MPSOperation(G.xgate(), 4)) - float(z["expect_x4"])) < 1e-5
    assert abs(m.expectation(MPSOperation(G.cnot(), (2, 3))) - float(z["expect_cnot23"])) < 1e-5
