"""Generate the golden fixtures under tests/golden/ (run once, in a container
that has the reference checkout; the fixtures travel, the reference does not).

  python tests/golden/make_golden.py --reference PATH_TO_MPSIM_CHECKOUT [--only NAME]

What it does:
1. Puts ``oracle/tn_shim`` (a restatement of the TensorNetwork 0.2.1 subset the
   reference calls, plus a one-function Cirq stub) on ``sys.path`` and applies
   two NumPy-2 compatibility patches the reference needs to import at all
   (``np.complex`` is gone, ``np.reshape`` lost its ``newshape=`` keyword).
2. Runs the reference's own unit tests (core_test.py, gates_test.py) against
   that shim and writes the outcome to ``reference_tests_under_shim.txt``:
   this checks the shim against the reference's known answers.
3. Runs seeded brickwork circuits through the reference's own, unmodified
   ``mpsim.core.MPS`` (complex64 gates = the plain reference; complex128 gates
   = the FP64 reference, which is what the reference does with its own
   complex128 Haar gates) and records, per two-qudit gate, every singular
   value TensorNetwork's SVD returned, the reference's own per-gate norm
   history (``MPS._norms``, core.py:1161), and final amplitudes.
4. Runs the same circuits through the NumPy oracle (oracle/ref_mps.py) and
   stores its results beside the reference's, so tests can check both.
5. For the 64-qubit workload, which the reference's per-gate norm sweep makes
   too slow to run through the reference, stores the oracle's results
   (complex64 and complex128) only.
6. ``observables.npz``: reduced density matrices, single-site marginals,
   seeded samples, ``from_wavefunction``, ``orthonormalize_*_edge_of``,
   non-unitary one-qudit gates and expectation values, all from the
   reference's own ``MPS`` on small seeded states (complex64).
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
SHIM = os.path.join(REPO, "oracle", "tn_shim")
sys.path.insert(0, REPO)

from mpsim_gb300 import circuits as C           # noqa: E402  (input generation)
from oracle.ref_mps import OracleMPS, canonical_spectra  # noqa: E402


def patch_numpy():
    """NumPy-2 shims the reference needs (applied only in this process)."""
    if not hasattr(np, "complex"):
        np.complex = complex
    orig = np.reshape

    def reshape(a, *args, **kw):
        if "newshape" in kw:
            kw["shape"] = kw.pop("newshape")
        return orig(a, *args, **kw)
    np.reshape = reshape


def import_reference(ref_root):
    sys.path.insert(0, SHIM)
    sys.path.insert(0, ref_root)
    patch_numpy()
    import tensornetwork as tn
    import mpsim.core as core
    return tn, core


class SvdRecorder:
    """Wraps the shim's svd_decomposition to record every full spectrum."""

    def __init__(self, tn):
        self.tn = tn
        self.spectra = []
        self.kept = []
        self._orig = tn.svd_decomposition

        def rec(tensor, split_axis, max_singular_values=None,
                max_truncation_error=None):
            u, s, vh, rest = self._orig(tensor, split_axis, max_singular_values,
                                        max_truncation_error)
            s_full = np.concatenate([np.asarray(s).real, np.asarray(rest).real])
            self.spectra.append(s_full.astype(np.float64))
            self.kept.append(int(s.shape[0]))
            return u, s, vh, rest
        tn.svd_decomposition = rec


def run_reference(core, tn, circ, dtype):
    rec = SvdRecorder(tn)
    mps = core.MPS(circ.nqudits, circ.d)
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for kind, sites, mat in circ.operations():
        g = np.asarray(mat).astype(dtype)
        if kind == 1:
            mps.apply_one_qudit_gate(tn.Node(g), sites[0])
        else:
            node = tn.Node(g.reshape((circ.d,) * 4))
            mps.apply_two_qudit_gate(node, sites[0], sites[1], **kw)
    tn.svd_decomposition = rec._orig
    return mps, rec


def run_oracle(circ, dtype):
    o = OracleMPS(circ.nqudits, circ.d, dtype)
    o.record = True
    kw = {} if circ.maxsvals is None else {"maxsvals": circ.maxsvals}
    for kind, sites, mat in circ.operations():
        if kind == 1:
            o.apply_one_qudit_gate(mat, sites[0])
        else:
            o.apply_two_qudit_gate(mat, sites[0], sites[1], **kw)
    return o


def pack_spectra(spectra, head=None):
    """Flatten per-gate spectra (optionally only the first ``head`` values)."""
    vals, offs = [], [0]
    for s in spectra:
        s = s if head is None else s[:head]
        vals.append(np.asarray(s, np.float64))
        offs.append(offs[-1] + len(s))
    return np.concatenate(vals) if vals else np.zeros(0), np.asarray(offs, np.int64)


def reference_amplitudes(core, mps, bits):
    """<x|psi> through the reference's own contraction (core.py:483-500)."""
    out = []
    d = mps.qudit_dimension
    for row in bits:
        other = core.MPS(mps.nqudits, d)
        for i, x in enumerate(row):
            if x:
                perm = np.zeros((d, d))
                perm[x, 0] = 1.0
                perm[0, x] = 1.0
                for k in range(1, d):
                    if k != x:
                        perm[k, k] = 1.0
                other.apply_one_qudit_gate(core.tn.Node(perm.astype(np.complex128)), i)
        # inner_product(self=mps, other=basis) = sum mps(x) conj(basis(x))
        out.append(mps.inner_product(other))
    return np.asarray(out, np.complex128)


def run_reference_unit_tests(ref_root):
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([SHIM, ref_root, os.path.join(HERE)])
    env["PYTHONDONTWRITEBYTECODE"] = "1"
    cmd = [sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider",
           "-p", "numpy2_compat", "--rootdir", HERE, "-c", os.devnull,
           os.path.join(ref_root, "mpsim", "core_test.py"),
           os.path.join(ref_root, "mpsim", "gates_test.py"), "-rA"]
    t0 = time.time()
    res = subprocess.run(cmd, env=env, capture_output=True, text=True, cwd=HERE)
    lines = [l for l in res.stdout.splitlines()
             if l.startswith(("PASSED", "FAILED", "ERROR"))]
    summary = res.stdout.strip().splitlines()[-1] if res.stdout.strip() else ""
    with open(os.path.join(HERE, "reference_tests_under_shim.txt"), "w") as f:
        f.write("# The reference's own unit tests (mpsim/core_test.py, gates_test.py)\n")
        f.write("# run unmodified against oracle/tn_shim (TensorNetwork 0.2.1 subset\n")
        f.write("# restated) with NumPy-2 compatibility patches.\n")
        f.write(f"# command: {' '.join(cmd[1:])}\n")
        f.write(f"# wall time {time.time() - t0:.1f}s; summary: {summary}\n")
        for l in sorted(lines):
            f.write(l.split(" - ")[0].replace("::", " ", 1) + "\n")
    print("reference unit tests under shim:", summary)


def golden_reference_circuit(core, tn, name, circ, nbits):
    out = {}
    bits = C.sample_bitstrings(circ.nqudits, circ.d, nbits, seed=1)
    out["bitstrings"] = bits.astype(np.int8)
    for tag, dt in (("c64", np.complex64), ("c128", np.complex128)):
        t0 = time.time()
        mps, rec = run_reference(core, tn, circ, dt)
        t_ref = time.time() - t0
        vals, offs = pack_spectra(rec.spectra)
        out[f"ref_{tag}_svals"] = vals
        out[f"ref_{tag}_offsets"] = offs
        out[f"ref_{tag}_kept"] = np.asarray(rec.kept, np.int64)
        out[f"ref_{tag}_norms"] = np.asarray(mps._norms, np.float64)
        out[f"ref_{tag}_bonds"] = np.asarray(mps.bond_dimensions(), np.int64)
        if circ.nqudits <= 12:
            out[f"ref_{tag}_wavefunction"] = np.asarray(mps.wavefunction(), np.complex128)
        out[f"ref_{tag}_amplitudes"] = reference_amplitudes(core, mps, bits)
        out[f"ref_{tag}_seconds"] = np.float64(t_ref)
        o = run_oracle(circ, dt)
        vals, offs = pack_spectra([h[0] for h in o.history])
        out[f"oracle_{tag}_svals"] = vals
        out[f"oracle_{tag}_offsets"] = offs
        out[f"oracle_{tag}_kept"] = np.asarray([h[1] for h in o.history], np.int64)
        out[f"oracle_{tag}_amplitudes"] = o.amplitudes(bits).astype(np.complex128)
        print(f"{name} {tag}: reference {t_ref:.1f}s, {len(rec.spectra)} two-qudit gates")
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def golden_oracle_circuit(name, circ, nbits, head=64):
    out = {}
    bits = C.sample_bitstrings(circ.nqudits, circ.d, nbits, seed=1)
    out["bitstrings"] = bits.astype(np.int8)
    for tag, dt in (("c64", np.complex64), ("c128", np.complex128)):
        t0 = time.time()
        o = run_oracle(circ, dt)
        vals, offs = pack_spectra([h[0] for h in o.history], head=head)
        out[f"oracle_{tag}_svals_head"] = vals.astype(np.float32)
        out[f"oracle_{tag}_offsets"] = offs
        out[f"oracle_{tag}_kept"] = np.asarray([h[1] for h in o.history], np.int64)
        out[f"oracle_{tag}_discarded"] = np.asarray([h[2] for h in o.history], np.float64)
        out[f"oracle_{tag}_norm"] = np.float64(o.norm())
        out[f"oracle_{tag}_amplitudes"] = o.amplitudes(bits).astype(np.complex128)
        spec = canonical_spectra(o)
        sv, so = pack_spectra(spec, head=head)
        out[f"oracle_{tag}_bond_spectra_head"] = sv.astype(np.float32)
        out[f"oracle_{tag}_bond_spectra_offsets"] = so
        out[f"oracle_{tag}_bonds"] = np.asarray(o.bond_dimensions(), np.int64)
        print(f"{name} {tag}: oracle {time.time() - t0:.1f}s")
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def known_answer_fixture(core, tn):
    """Small cases from the reference's tests, run through the reference."""
    from mpsim import gates as G
    cases = {}
    # Bell with maxsvals=1 (core_test.py:1084-1091, 1123-1134)
    m = core.MPS(2)
    m.h(0)
    m.cnot(0, 1, maxsvals=1)
    cases["bell_maxsvals1"] = m.wavefunction()
    # GHZ with non-local CNOTs (core_test.py:1236-1245)
    m = core.MPS(5)
    m.h(0)
    for i in range(1, 5):
        m.cnot(0, i)
    cases["ghz5_nonlocal"] = m.wavefunction()
    # QFT on 4 qubits (core_test.py:1248-1258)
    m = core.MPS(4)
    for i in range(3, -1, -1):
        m.h(i)
        for j in range(i - 1, -1, -1):
            m.apply_two_qudit_gate(G.cphase(2 ** (j - i)), j, i)
    cases["qft4"] = m.wavefunction()
    # fraction truncation (core_test.py:915-922)
    m = core.MPS(2)
    m.h(0)
    m.cnot(0, 1, fraction=0.5)
    cases["bell_fraction_half"] = m.wavefunction()
    # right-canonical CNOT chain on qutrits with a Haar gate
    m = core.MPS(4, 3)
    for i in range(4):
        m.apply_one_qudit_gate(tn.Node(C.haar_random_matrix(1, 3, 11 + i)), i)
    for (a, b) in [(0, 1), (2, 3), (1, 2), (2, 1), (0, 1)]:
        g = C.haar_random_matrix(2, 3, 100 + a * 7 + b).reshape(3, 3, 3, 3)
        m.apply_two_qudit_gate(tn.Node(g), a, b, keep_left_canonical=(a != 2))
    cases["qutrit4_mixed"] = m.wavefunction()
    np.savez_compressed(os.path.join(HERE, "known_answers.npz"),
                        **{k: np.asarray(v, np.complex128) for k, v in cases.items()})
    print("known answers:", ", ".join(cases))


# Small seeded states for the observables fixture: (name, nqudits, d, depth,
# maxsvals, seed).  The GPU tests rebuild them from the same circuits.
OBS_STATES = [("q6", 6, 2, 3, None, 21), ("t4", 4, 3, 2, None, 22), ("q8trunc", 8, 2, 5, 3, 23)]
OBS_RDM = {"q6": [(0,), (3,), (1, 2), (4, 1), (0, 5, 2)], "t4": [(1,), (0, 3), (2, 1)],
           "q8trunc": [(2,), (5, 6)]}


def observables_fixture(core, tn):
    """Row (f) functions of the reference, run through the reference."""
    from mpsim import gates as G
    out = {}

    def build(n, d, depth, maxsvals, seed):
        circ = C.brickwork(n, depth, d=d, maxsvals=maxsvals, seed=seed)
        m = core.MPS(n, d)
        kw = {} if maxsvals is None else {"maxsvals": maxsvals}
        for kind, sites, mat in circ.operations():
            g = np.asarray(mat).astype(np.complex64)
            if kind == 1:
                m.apply_one_qudit_gate(tn.Node(g), sites[0])
            else:
                m.apply_two_qudit_gate(tn.Node(g.reshape((d,) * 4)), sites[0], sites[1], **kw)
        return m

    states = {}
    for name, n, d, depth, maxs, seed in OBS_STATES:
        m = build(n, d, depth, maxs, seed)
        states[name] = m
        out[f"{name}_wf"] = m.wavefunction()
        for idx in OBS_RDM[name]:
            key = "_".join(str(i) for i in idx)
            out[f"{name}_rdm_{key}"] = m.reduced_density_matrix(list(idx))
        out[f"{name}_marginals"] = np.stack(
            [m.reduced_density_matrix(i).diagonal().real for i in range(n)])
    # seeded samples (the normalised states only: a truncated state's
    # marginals do not sum to one and np.random.choice refuses them)
    np.random.seed(7)
    out["q6_samples"] = np.asarray(states["q6"].sample(25), dtype=np.int64)
    np.random.seed(8)
    hist = states["q6"].sample(40, as_hist=True)
    out["q6_hist_keys"] = np.asarray(sorted(hist))
    out["q6_hist_counts"] = np.asarray([hist[k] for k in sorted(hist)], dtype=np.int64)
    np.random.seed(9)
    out["t4_samples"] = np.asarray(states["t4"].sample(20, as_string=True))
    # from_wavefunction
    rng = np.random.default_rng(31)
    for name, n, d in (("fw_q6", 6, 2), ("fw_t4", 4, 3)):
        psi = (rng.normal(size=d ** n) + 1j * rng.normal(size=d ** n)).astype(np.complex64)
        psi /= np.linalg.norm(psi)
        m = core.MPS.from_wavefunction(psi, n, d)
        out[f"{name}_psi"] = psi
        out[f"{name}_wf"] = m.wavefunction()
        out[f"{name}_bonds"] = np.asarray(m.bond_dimensions())
    # orthonormalisation of one edge
    m = build(6, 2, 3, None, 21)
    m.orthonormalize_right_edge_of(2)
    out["ortho_r2_wf"], out["ortho_r2_bonds"] = m.wavefunction(), np.asarray(m.bond_dimensions())
    m.orthonormalize_left_edge_of(4)
    out["ortho_l4_wf"], out["ortho_l4_bonds"] = m.wavefunction(), np.asarray(m.bond_dimensions())
    # non-unitary gates: a projector on a GHZ state (exact zero singular
    # values: orthonormalisation must cut the bonds to 1), and a general
    # non-unitary gate with each keyword combination
    m = core.MPS(4)
    m.h(0)
    for i in range(3):
        m.cnot(i, i + 1)
    m.apply_one_qudit_gate(G.computational_basis_projector(0), 1)
    out["ghz_proj_wf"], out["ghz_proj_bonds"] = m.wavefunction(), np.asarray(m.bond_dimensions())
    damp = np.array([[1.0, 0.0], [0.0, 0.4]], dtype=np.complex64)
    for tag, kw in (("default", {}), ("noortho", {"ortho_after_non_unitary": False}),
                    ("norenorm", {"renormalize_after_non_unitary": False}), ("end", {})):
        m = build(6, 2, 3, None, 21)
        site = 5 if tag == "end" else 3
        m.apply_one_qudit_gate(tn.Node(damp), site, **kw)
        out[f"nonunit_{tag}_wf"] = m.wavefunction()
        out[f"nonunit_{tag}_bonds"] = np.asarray(m.bond_dimensions())
        out[f"nonunit_{tag}_norm"] = np.float64(m.norm())
    # expectation values
    m = states["q6"]
    out["expect_z1"] = np.float64(m.expectation(core.MPSOperation(G.zgate(), 1)))
    out["expect_x4"] = np.float64(m.expectation(core.MPSOperation(G.xgate(), 4)))
    out["expect_cnot23"] = np.float64(m.expectation(core.MPSOperation(G.cnot(), (2, 3))))
    np.savez_compressed(os.path.join(HERE, "observables.npz"), **out)
    print("observables:", len(out), "arrays")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="root of a grmlarose/mpsim checkout (the directory holding mpsim/)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    only = args.only
    if only in (None, "unit"):
        run_reference_unit_tests(args.reference)
    tn, core = import_reference(args.reference)
    core.tn = tn
    if only in (None, "kat"):
        known_answer_fixture(core, tn)
    if only in (None, "cfg0"):
        golden_reference_circuit(core, tn, "brickwork_10q_d10_full",
                                 C.workload("brickwork_10q_d10_full"), 256)
    if only in (None, "cfg0q"):
        golden_reference_circuit(core, tn, "brickwork_8qutrit_d8_chi12",
                                 C.brickwork(8, 8, d=3, maxsvals=12, seed=3), 256)
    if only in (None, "cfg1"):
        golden_reference_circuit(core, tn, "brickwork_48q_d24_chi128",
                                 C.workload("brickwork_48q_d24_chi128"), 64)
    if only in (None, "obs"):
        observables_fixture(core, tn)
    if only in (None, "cfg2"):
        golden_oracle_circuit("brickwork_64q_d40_chi256",
                              C.workload("brickwork_64q_d40_chi256"), 64)


if __name__ == "__main__":
    main()
