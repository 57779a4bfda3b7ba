"""NumPy restatement of mpsim's MPS gate-application path (the oracle).

Test infrastructure: only tests, ``smoke()`` and the CPU-baseline legs of
``bench.py`` use this module.  It restates, in plain NumPy, what the reference
computes through TensorNetwork 0.2.1 and LAPACK:

* ``OracleMPS.__init__``            mpsim/core.py:161-243 (|0...0> product state,
                                     max bond dimensions d**min(k+1, n-1-k)).
* ``OracleMPS.apply_one_qudit_gate`` mpsim/core.py:753-826 (unitary branch:
                                     gate edge 1 contracts with the site).
* ``OracleMPS.apply_two_qudit_gate`` mpsim/core.py:950-1161: index flip
                                     (1030-1033), swap network for non-adjacent
                                     sites (1035-1043, 1154-1158), merge
                                     (1059-1062), gate contraction (1064-1068),
                                     ``fraction``/``maxsvals`` (1104-1130),
                                     truncated SVD via TensorNetwork's
                                     ``split_node_full_svd`` (1132-1137, which
                                     calls ``np.linalg.svd(full_matrices=False)``
                                     and keeps ``s[:max_singular_values]``),
                                     S placement (1139-1145).
* ``wavefunction``                  mpsim/core.py:483-500 (big-endian).
* ``inner_product`` / ``norm``      mpsim/core.py:507-565 (conj on *other*).
* ``renormalize``                   mpsim/core.py:567-594.
* ``reduced_density_matrix``        mpsim/core.py:596-653 (ket digits of the
                                     kept sites in the given order, then bra).
* ``site_marginals`` / ``sample``   mpsim/core.py:655-709 (each digit drawn
                                     from that site's marginal of the
                                     unconditioned state).
* ``from_wavefunction``             mpsim/core.py:245-328 (split_node at every
                                     cut, nothing truncated, sqrt(S) on both
                                     sides).
* ``orthonormalize_*_edge_of``      mpsim/core.py:847-937 (split_node_full_svd
                                     with max_truncation_err = threshold*norm).
* non-unitary one-qudit gates       mpsim/core.py:793-845.
* ``haar_random_unitary``           mpsim/gates.py:248-286 (Mezzadri QR).

Site tensors are stored as (chi_left, d, chi_right) arrays.  The reference
orders axes as TensorNetwork leaves them; only gauge-invariant quantities
(singular values, amplitudes, norms, overlaps) are compared, so the axis order
is free.  ``dtype`` selects complex64 (gates cast to complex64 first, the
"plain" reference) or complex128 (the FP64 oracle).
"""

from __future__ import annotations

import numpy as np


def haar_random_unitary(nqudits=2, qudit_dimension=2, seed=None):
    """mpsim/gates.py:248-286: Q of QR of a complex Gaussian, phase-fixed."""
    rng = np.random.RandomState(seed)
    units = np.array([1, 1j])
    dim = qudit_dimension ** nqudits
    mat = np.sum(rng.randn(dim, dim, 2) * units, axis=-1) / np.sqrt(2)
    q, r = np.linalg.qr(mat)
    diag = np.diag(r).copy()
    diag /= np.abs(diag)
    return np.reshape(q * diag, [qudit_dimension] * 2 * nqudits)


def kept_count(maxsvals, rank):
    """Number of singular values TensorNetwork keeps for ``max_singular_values``.

    TensorNetwork slices ``s[:max_singular_values]`` after clamping with
    ``min``; a negative value therefore behaves like a Python slice stop.
    """
    if maxsvals is None:
        return rank
    return len(range(rank)[:min(int(maxsvals), rank)])


class OracleMPS:
    """Matrix product state with the reference's semantics, in NumPy."""

    def __init__(self, nqudits, qudit_dimension=2, dtype=np.complex64):
        if nqudits < 2:
            raise ValueError(
                f"Number of qudits must be greater than 2 but is {nqudits}.")
        self.n = nqudits
        self.d = qudit_dimension
        self.dtype = np.dtype(dtype)
        self.sites = []
        for _ in range(nqudits):
            t = np.zeros((1, qudit_dimension, 1), dtype=self.dtype)
            t[0, 0, 0] = 1.0
            self.sites.append(t)
        half = [qudit_dimension ** (i + 1) for i in range(nqudits // 2)]
        maxb = half + list(reversed(half))
        if nqudits % 2 == 0:
            maxb.remove(qudit_dimension ** (nqudits // 2))
        self.max_bond_dimensions = maxb
        # Per two-qudit gate: (all singular values, kept count, discarded
        # weight).  Filled only when ``record`` is True.
        self.record = False
        self.history = []

    # -- structure ---------------------------------------------------------
    def bond_dimensions(self):
        return [self.sites[i].shape[2] for i in range(self.n - 1)]

    def max_bond_dimension_of(self, edge_index):
        if edge_index >= self.n:
            raise ValueError(
                f"Edge index should be less than {self.n} but is {edge_index}.")
        return self.max_bond_dimensions[edge_index]

    def copy(self):
        new = OracleMPS(self.n, self.d, self.dtype)
        new.sites = [s.copy() for s in self.sites]
        return new

    # -- gates -------------------------------------------------------------
    def apply_one_qudit_gate(self, gate, i, renormalize_after_non_unitary=True,
                             ortho_after_non_unitary=True):
        u = np.asarray(gate).astype(self.dtype)
        unitary = bool(np.allclose(u.conj().T @ u, np.identity(u.shape[0]), atol=1e-5))
        norm = self.norm() if (not unitary and renormalize_after_non_unitary) else None
        s = self.sites[i]
        # new[l, a', r] = sum_a U[a', a] s[l, a, r]   (core.py:820-826)
        self.sites[i] = np.einsum("xa,lar->lxr", u, s).astype(self.dtype)
        if not unitary and ortho_after_non_unitary:   # core.py:828-842
            if i == 0:
                self.orthonormalize_right_edge_of(i)
            elif i == self.n - 1:
                self.orthonormalize_left_edge_of(i)
            else:
                self.orthonormalize_right_edge_of(i)
                self.orthonormalize_left_edge_of(i)
        if norm is not None:                          # core.py:844-845
            self.renormalize(norm)

    @staticmethod
    def _kept_by_error(s, max_err):
        """split_node_full_svd's max_truncation_err rule (TensorNetwork
        0.2.1): count of sqrt(cumsum(s[::-1]^2)) above the bound."""
        errs = np.sqrt(np.cumsum(np.square(s[::-1])))
        return int(np.count_nonzero(errs > max_err))

    def orthonormalize_right_edge_of(self, i, threshold=1e-8):
        """core.py:847-891: SVD with rows (digit, left bond), site <- U,
        right neighbour <- S V^H . neighbour."""
        if not 0 <= i < self.n - 1:
            raise ValueError("Invalid edge index.")
        a = self.sites[i]
        chil, d, chir = a.shape
        max_err = threshold * self.norm()
        u, s, vh = np.linalg.svd(a.reshape(chil * d, chir), full_matrices=False)
        k = self._kept_by_error(s, max_err)
        right = (s[:k].astype(self.dtype)[:, None] * vh[:k]).astype(self.dtype)
        nxt = self.sites[i + 1]
        self.sites[i] = np.ascontiguousarray(u[:, :k].reshape(chil, d, k))
        self.sites[i + 1] = (right @ nxt.reshape(chir, -1)).reshape(k, d, nxt.shape[2])

    def orthonormalize_left_edge_of(self, i, threshold=1e-8):
        """core.py:893-937: SVD with columns (digit, right bond), site <-
        V^H, left neighbour <- neighbour . U S."""
        if not 0 < i <= self.n - 1:
            raise ValueError("Invalid edge index.")
        a = self.sites[i]
        chil, d, chir = a.shape
        max_err = threshold * self.norm()
        u, s, vh = np.linalg.svd(a.reshape(chil, d * chir), full_matrices=False)
        k = self._kept_by_error(s, max_err)
        left = (u[:, :k] * s[:k].astype(self.dtype)[None, :]).astype(self.dtype)
        prev = self.sites[i - 1]
        self.sites[i] = np.ascontiguousarray(vh[:k].reshape(k, d, chir))
        self.sites[i - 1] = (prev.reshape(-1, chil) @ left).reshape(prev.shape[0], d, k)

    @staticmethod
    def from_wavefunction(psi, nqudits, qudit_dimension=2, dtype=np.complex64):
        """core.py:245-328: split at every cut with TensorNetwork's
        split_node (full SVD, nothing truncated, sqrt(S) on both sides)."""
        d = qudit_dimension
        o = OracleMPS(nqudits, d, dtype)
        rest = np.asarray(psi).astype(o.dtype).reshape(1, -1)
        chi = 1
        sites = []
        for i in range(nqudits - 1):
            mat = rest.reshape(chi * d, -1)
            u, s, vh = np.linalg.svd(mat, full_matrices=False)
            sq = np.sqrt(s).astype(o.dtype)
            k = s.size
            sites.append((u * sq[None, :]).reshape(chi, d, k))
            rest = sq[:, None] * vh
            chi = k
        sites.append(rest.reshape(chi, d, 1))
        o.sites = [np.ascontiguousarray(t) for t in sites]
        return o

    def apply_two_qudit_gate(self, gate, i, j, **kwargs):
        g = np.asarray(gate).astype(self.dtype).reshape((self.d,) * 4)
        if i == j:
            raise ValueError("Node indices cannot be identical.")
        if j < i:                                   # core.py:1030-1033
            g = g.transpose(1, 0, 3, 2)
            i, j = j, i
        invert = False
        if i < j - 1:                               # core.py:1035-1043
            invert = True
            original = i
            for a in range(i, j - 1):
                self.swap(a, a + 1, **kwargs)
            i = j - 1
        maxsvals = self._parse_truncation(i, j, kwargs)
        left_canonical = kwargs.get("keep_left_canonical", True) \
            if "keep_left_canonical" in kwargs else True
        self._apply_adjacent(g, i, maxsvals, left_canonical)
        if invert:                                  # core.py:1154-1158
            cur = i
            while cur > original:
                self.swap(cur - 1, cur, **kwargs)
                cur -= 1

    def _parse_truncation(self, i, j, kwargs):
        """core.py:1110-1130 (uses the indices after the swap network)."""
        if "fraction" in kwargs and "maxsvals" in kwargs:
            raise ValueError(
                "Only one of (fraction, maxsvals) can be provided as kwargs.")
        maxsvals = None
        if "fraction" in kwargs:
            fraction = kwargs["fraction"]
            if not (0 <= fraction <= 1):
                raise ValueError("Keyword fraction must be between 0 and 1")
            maxsvals = int(round(fraction * self.max_bond_dimension_of(min(i, j))))
        if "maxsvals" in kwargs:
            maxsvals = int(kwargs["maxsvals"])
        return maxsvals

    def _apply_adjacent(self, g, i, maxsvals, left_canonical):
        a, b = self.sites[i], self.sites[i + 1]
        chil, d, chim = a.shape
        chir = b.shape[2]
        # merge (core.py:1059-1062) then gate (core.py:1064-1068)
        m = (a.reshape(chil * d, chim) @ b.reshape(chim, d * chir))
        m = m.reshape(chil, d, d, chir)
        theta = np.einsum("xyab,labr->lxyr", g, m).astype(self.dtype)
        theta = theta.reshape(chil * d, d * chir)
        # split_node_full_svd (core.py:1132-1137)
        u, s, vh = np.linalg.svd(theta, full_matrices=False)
        k = kept_count(maxsvals, s.size)
        if self.record:
            s64 = s.astype(np.float64)
            self.history.append((s64.copy(), k, float(np.sum(s64[k:] ** 2))))
        sk = s[:k].astype(self.dtype)
        u, vh = u[:, :k], vh[:k, :]
        if left_canonical:                          # core.py:1139-1145
            left, right = u, sk[:, None] * vh
        else:
            left, right = u * sk[None, :], vh
        self.sites[i] = np.ascontiguousarray(left.reshape(chil, d, k))
        self.sites[i + 1] = np.ascontiguousarray(right.reshape(k, d, chir))

    def swap(self, a, b, **kwargs):
        """core.py:1376-1380 with the SWAP matrix of gates.py:204-212."""
        if b < a:
            a, b = b, a
        sw = np.zeros((self.d ** 2, self.d ** 2))
        for x in range(self.d):
            for y in range(self.d):
                sw[y * self.d + x, x * self.d + y] = 1.0
        self.apply_two_qudit_gate(sw, a, b, **kwargs)

    # -- contractions ------------------------------------------------------
    def wavefunction(self):
        """core.py:483-500: left-to-right chain, qudit 0 most significant."""
        psi = np.ones((1, 1), dtype=self.dtype)
        for s in self.sites:
            chil, d, chir = s.shape
            psi = (psi @ s.reshape(chil, d * chir)).reshape(-1, chir)
        return psi.reshape(-1)

    def inner_product(self, other):
        """core.py:507-561: sum_x self(x) * conj(other(x))."""
        if other.n != self.n:
            raise ValueError("Number of qudits must be equal.")
        if other.d != self.d:
            raise ValueError("Qudit dimensions must be equal.")
        env = np.ones((1, 1), dtype=np.result_type(self.dtype, other.dtype))
        for a, b in zip(self.sites, other.sites):
            # env[l, l'] a[l, x, r] conj(b)[l', x, r'] -> env'[r, r']
            t = np.tensordot(env, np.conj(b), axes=([1], [0]))   # l, x, r'
            env = np.tensordot(a, t, axes=([0, 1], [0, 1]))      # r, r'
        return complex(env[0, 0])

    def norm(self):
        """core.py:563-565."""
        return float(np.sqrt(self.inner_product(self).real))

    def renormalize(self, to_norm=1.0):
        """core.py:567-594."""
        if to_norm < 0.0:
            raise ValueError(f"Arg to_norm must be positive but is {to_norm}")
        if np.isclose(to_norm, 0.0, atol=1e-15):
            raise ValueError(f"Arg to_norm = {to_norm} is too close to numerical zero.")
        norm = self.norm()
        if np.isclose(norm, 0.0, atol=1e-15):
            raise ValueError("Norm of MPS is numerically zero, cannot renormalize.")
        factor = (to_norm / norm) ** (1 / self.n)
        self.sites = [(factor * s).astype(self.dtype) for s in self.sites]

    def reduced_density_matrix(self, node_indices):
        """core.py:596-653: rho[(ket digits of node_indices in the given
        order), (bra digits)], the other sites traced out, not normalised."""
        try:
            node_indices = tuple(iter(node_indices))
        except TypeError:
            node_indices = (node_indices,)
        kept = sorted(node_indices)
        d = self.d
        # env[b, l, l'] with b = (a_1, a_1', a_2, a_2', ...) over kept sites
        env = np.ones((1, 1, 1), dtype=self.dtype)
        for i, s in enumerate(self.sites):
            f = np.einsum("bkl,kar->blar", env, s)            # b, l', a, r
            if i in kept:
                env = np.einsum("blar,lcs->bacrs", f, np.conj(s))
                env = env.reshape(-1, s.shape[2], s.shape[2])
            else:
                env = np.einsum("blar,las->brs", f, np.conj(s))
        k = len(kept)
        vals = env.reshape((d,) * (2 * k))
        pos = {site: p for p, site in enumerate(kept)}
        perm = [2 * pos[i] for i in node_indices] + [2 * pos[i] + 1 for i in node_indices]
        return np.ascontiguousarray(vals.transpose(perm)).reshape(d ** k, d ** k)

    def site_marginals(self):
        """reduced_density_matrix(i).diagonal().real for every site
        (core.py:661), as float of the state's precision."""
        real = np.float32 if self.dtype == np.complex64 else np.float64
        return np.stack([self.reduced_density_matrix(i).diagonal().real.astype(real)
                         for i in range(self.n)])

    def sample(self, nsamples, as_hist=False, as_string=False):
        """core.py:655-709: per sample and site, np.random.choice over the
        digits with that site's marginal (global NumPy RNG)."""
        if as_hist:
            as_string = True
        probs = self.site_marginals()
        states = list(range(self.d))
        raw = []
        for _ in range(nsamples):
            string = [np.random.choice(states, size=1, p=probs[i])[0] for i in range(self.n)]
            raw.append("".join(str(b) for b in string) if as_string else string)
        if as_hist:
            hist = {}
            for b in raw:
                hist[b] = hist.get(b, 0) + 1
            return hist
        return raw

    def amplitudes(self, bitstrings):
        """<x|psi> for each row x of ``bitstrings`` (shape (S, n))."""
        bits = np.asarray(bitstrings)
        nb = bits.shape[0]
        env = np.ones((nb, 1), dtype=self.dtype)
        for i, s in enumerate(self.sites):
            new = np.zeros((nb, s.shape[2]), dtype=self.dtype)
            for x in range(self.d):
                rows = bits[:, i] == x
                if np.any(rows):
                    new[rows] = env[rows] @ s[:, x, :]
            env = new
        return env[:, 0]


def canonical_spectra(mps):
    """Schmidt spectra of every bond of the normalised-or-not state.

    A left-to-right QR sweep brings the state to left-canonical form; a
    right-to-left SVD sweep then reads each bond's Schmidt coefficients.
    These are gauge-invariant, so two MPS of the same state agree on them.
    Returned in float64, descending, one array per bond.
    """
    sites = [s.astype(np.complex128) for s in mps.sites]
    n = len(sites)
    for i in range(n - 1):
        chil, d, chir = sites[i].shape
        q, r = np.linalg.qr(sites[i].reshape(chil * d, chir))
        sites[i] = q.reshape(chil, d, q.shape[1])
        sites[i + 1] = np.tensordot(r, sites[i + 1], axes=([1], [0]))
    spectra = [None] * (n - 1)
    for i in range(n - 1, 0, -1):
        chil, d, chir = sites[i].shape
        u, s, vh = np.linalg.svd(sites[i].reshape(chil, d * chir),
                                 full_matrices=False)
        spectra[i - 1] = s
        sites[i] = vh.reshape(vh.shape[0], d, chir)
        sites[i - 1] = np.tensordot(sites[i - 1], u * s[None, :], axes=([2], [0]))
    return spectra


def overlap_infidelity(a, b):
    """1 - |<a|b>|^2 / (<a|a><b|b>) from MPS overlaps (complex128 sweep)."""
    a64, b64 = a.copy(), b.copy()
    a64.sites = [s.astype(np.complex128) for s in a.sites]
    b64.sites = [s.astype(np.complex128) for s in b.sites]
    a64.dtype = b64.dtype = np.dtype(np.complex128)
    ab = a64.inner_product(b64)
    aa = a64.inner_product(a64).real
    bb = b64.inner_product(b64).real
    return float(1.0 - abs(ab) ** 2 / (aa * bb))
