"""The NumPy oracle's observables, splits and non-unitary gates against the
reference's own outputs (CPU).

tests/golden/observables.npz holds what the reference's unmodified
mpsim/core.py returned (through tests/golden/make_golden.py) for
reduced_density_matrix, the sampling marginals and seeded draws,
from_wavefunction, orthonormalize_*_edge_of, non-unitary one-qudit gates and
expectation values on small seeded states, all in complex64.
"""
import importlib.util
import os

import numpy as np
import pytest

from oracle.ref_mps import OracleMPS
from mpsim_gb300 import circuits as C
from mpsim_gb300 import gates as G

from conftest import GOLDEN

_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)
STATES = {s[0]: s[1:] for s in make_golden.OBS_STATES}
RDM = make_golden.OBS_RDM


@pytest.fixture(scope="module")
def z():
    return np.load(os.path.join(GOLDEN, "observables.npz"))


def oracle_state(name):
    n, d, depth, maxs, seed = STATES[name]
    circ = C.brickwork(n, depth, d=d, maxsvals=maxs, seed=seed)
    o = OracleMPS(n, d, np.complex64)
    kw = {} if maxs is None else {"maxsvals": maxs}
    for kind, sites, mat in circ.operations():
        if kind == 1:
            o.apply_one_qudit_gate(mat, sites[0])
        else:
            o.apply_two_qudit_gate(mat, sites[0], sites[1], **kw)
    return o


@pytest.mark.parametrize("name", list(STATES))
def test_oracle_rdm_and_marginals(z, name):
    o = oracle_state(name)
    assert np.allclose(o.wavefunction(), z[f"{name}_wf"], atol=2e-6)
    for idx in RDM[name]:
        key = "_".join(str(i) for i in idx)
        assert np.allclose(o.reduced_density_matrix(idx), z[f"{name}_rdm_{key}"], atol=2e-6), idx
    assert np.allclose(o.site_marginals(), z[f"{name}_marginals"], atol=2e-6)


def test_oracle_samples_equal_reference_draws(z):
    q6 = oracle_state("q6")
    np.random.seed(7)
    assert np.array_equal(np.asarray(q6.sample(25)), z["q6_samples"])
    np.random.seed(8)
    hist = q6.sample(40, as_hist=True)
    assert sorted(hist) == list(z["q6_hist_keys"])
    assert [hist[k] for k in sorted(hist)] == list(z["q6_hist_counts"])
    np.random.seed(9)
    assert list(oracle_state("t4").sample(20, as_string=True)) == list(z["t4_samples"])


@pytest.mark.parametrize("name,n,d", [("fw_q6", 6, 2), ("fw_t4", 4, 3)])
def test_oracle_from_wavefunction(z, name, n, d):
    o = OracleMPS.from_wavefunction(z[f"{name}_psi"], n, d)
    assert np.allclose(o.wavefunction(), z[f"{name}_wf"], atol=2e-6)
    assert list(o.bond_dimensions()) == list(z[f"{name}_bonds"])


def test_oracle_orthonormalize(z):
    o = oracle_state("q6")
    o.orthonormalize_right_edge_of(2)
    assert np.allclose(o.wavefunction(), z["ortho_r2_wf"], atol=2e-6)
    assert list(o.bond_dimensions()) == list(z["ortho_r2_bonds"])
    o.orthonormalize_left_edge_of(4)
    assert np.allclose(o.wavefunction(), z["ortho_l4_wf"], atol=2e-6)
    assert list(o.bond_dimensions()) == list(z["ortho_l4_bonds"])
    with pytest.raises(ValueError):
        o.orthonormalize_right_edge_of(5)
    with pytest.raises(ValueError):
        o.orthonormalize_left_edge_of(0)


def test_oracle_non_unitary_gates(z):
    # projector on a GHZ state: exact zero singular values, bonds cut to 1
    o = OracleMPS(4, 2, np.complex64)
    o.apply_one_qudit_gate(G.hgate().tensor, 0)
    for i in range(3):
        o.apply_two_qudit_gate(G.cnot().tensor.reshape(4, 4), i, i + 1)
    o.apply_one_qudit_gate(G.computational_basis_projector(0).tensor, 1)
    assert np.allclose(o.wavefunction(), z["ghz_proj_wf"], atol=2e-6)
    assert list(o.bond_dimensions()) == list(z["ghz_proj_bonds"])
    damp = np.array([[1.0, 0.0], [0.0, 0.4]])
    for tag, kw in (("default", {}), ("noortho", {"ortho_after_non_unitary": False}),
                    ("norenorm", {"renormalize_after_non_unitary": False}), ("end", {})):
        o = oracle_state("q6")
        o.apply_one_qudit_gate(damp, 5 if tag == "end" else 3, **kw)
        assert np.allclose(o.wavefunction(), z[f"nonunit_{tag}_wf"], atol=2e-6), tag
        assert list(o.bond_dimensions()) == list(z[f"nonunit_{tag}_bonds"]), tag
        assert abs(o.norm() - float(z[f"nonunit_{tag}_norm"])) < 2e-6, tag


def test_oracle_expectation_values(z):
    psi = oracle_state("q6").wavefunction().astype(np.complex128).reshape((2,) * 6)

    def expect(op, sites):
        k = len(sites)
        u = np.asarray(op, np.complex128).reshape((2,) * (2 * k))
        phi = np.tensordot(u, psi, axes=(list(range(k, 2 * k)), list(sites)))
        phi = np.moveaxis(phi, list(range(k)), list(sites))
        return float(np.vdot(psi, phi).real)
    assert abs(expect(G.zgate().tensor, [1]) - float(z["expect_z1"])) < 1e-5
    assert abs(expect(G.xgate().tensor, [4]) - float(z["expect_x4"])) < 1e-5
    assert abs(expect(G.cnot().tensor, [2, 3]) - float(z["expect_cnot23"])) < 1e-5
