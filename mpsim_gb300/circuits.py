"""Seeded synthetic brickwork circuits (the benchmark and parity workloads).

Every gate is drawn by ``haar_random_matrix`` (mpsim/gates.py:248-286) with an
explicit 32-bit seed derived from (base seed, instance, layer, slot, kind), so
any single gate of any circuit can be regenerated on its own.  Layer t applies
a one-qudit Haar U(d) to every site, then two-qudit Haar U(d^2) gates on the
pairs (2j, 2j+1) for even t and (2j+1, 2j+2) for odd t.

Workloads (qubit count, depth, truncation) named by their sizes:
  brickwork_10q_d10_full     10 qubits, depth 10, no truncation
  brickwork_48q_d24_chi128   48 qubits, depth 24, maxsvals=128
  brickwork_64q_d40_chi256   64 qubits, depth 40, maxsvals=256 (theta 512x512)
  batch_512_mixed            512 circuits, 16-48 qubits, depth 8-32,
                             maxsvals in {16,32,64,128}, 20% CNOT/CZ slots
  qutrit_128x32_d30_chi192   128 circuits of 32 qutrits, depth 30, maxsvals=192
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .gates import haar_random_matrix, _cnot_matrix

KIND_1Q = 1
KIND_2Q = 2


def gate_seed(base: int, instance: int, layer: int, slot: int, kind: int) -> int:
    """32-bit RandomState seed for one gate."""
    ss = np.random.SeedSequence([base, instance, layer, slot, kind])
    return int(ss.generate_state(1, dtype=np.uint32)[0])


def gate_seeds(base: int, instance: int, layer: int, slots, kind: int) -> List[int]:
    """gate_seed for many slots of one layer."""
    return [gate_seed(base, instance, layer, int(i), kind) for i in slots]


def haar_batch(nqudits: int, d: int, seeds: Sequence[int]) -> np.ndarray:
    """haar_random_matrix(nqudits, d, seed) for every seed, stacked: the same
    RandomState draws, one stacked QR (NumPy factorises each matrix with the
    same LAPACK call as for a single one, so every gate is identical) and the
    same phase fix."""
    dim = d ** nqudits
    if len(seeds) == 0:
        return np.zeros((0, dim, dim), np.complex128)
    z = np.stack([np.random.RandomState(s).randn(dim, dim, 2) for s in seeds])
    mat = (z[..., 0] + 1j * z[..., 1]) / np.sqrt(2)
    q, r = np.linalg.qr(mat)
    ph = np.diagonal(r, axis1=1, axis2=2).copy()
    ph /= np.abs(ph)
    return q * ph[:, None, :]


@dataclass
class Layer:
    one_q: np.ndarray              # (n, d, d) complex128: U[a', a] per site
    pair_left: np.ndarray          # (p,) int: left site of each pair
    two_q: np.ndarray              # (p, d*d, d*d) complex128: U[(a'b'),(ab)]


@dataclass
class BrickworkCircuit:
    nqudits: int
    d: int
    depth: int
    maxsvals: Optional[int]
    seed: int = 0
    instance: int = 0
    layers: List[Layer] = field(default_factory=list)

    @property
    def n_two_qudit_gates(self) -> int:
        return int(sum(len(l.pair_left) for l in self.layers))

    @property
    def n_one_qudit_gates(self) -> int:
        return int(sum(l.one_q.shape[0] for l in self.layers))

    def operations(self):
        """Gates in application order as (kind, sites, matrix)."""
        for lay in self.layers:
            for i in range(self.nqudits):
                yield (1, (i,), lay.one_q[i])
            for p, i in enumerate(lay.pair_left):
                yield (2, (int(i), int(i) + 1), lay.two_q[p])


def brickwork(nqudits: int, depth: int, d: int = 2, maxsvals: Optional[int] = None,
              seed: int = 0, instance: int = 0, special_fraction: float = 0.0
              ) -> BrickworkCircuit:
    """Seeded brickwork circuit; ``special_fraction`` of the two-qudit slots
    (qubits only) hold a fixed CNOT or CZ instead of a Haar unitary."""
    circ = BrickworkCircuit(nqudits, d, depth, maxsvals, seed, instance)
    pick = np.random.default_rng(np.random.SeedSequence([seed, instance, 7919]))
    cz = np.diag([1, 1, 1, -1]).astype(np.complex128)
    cn = _cnot_matrix.reshape(4, 4).astype(np.complex128)
    for t in range(depth):
        one = haar_batch(1, d, gate_seeds(seed, instance, t, range(nqudits), KIND_1Q))
        start = t % 2
        lefts = np.arange(start, nqudits - 1, 2, dtype=np.int64)
        special = {}
        for i in lefts:
            if special_fraction > 0 and pick.random() < special_fraction:
                special[int(i)] = cn if pick.random() < 0.5 else cz
        haar_slots = [int(i) for i in lefts if int(i) not in special]
        haar = haar_batch(2, d, gate_seeds(seed, instance, t, haar_slots, KIND_2Q))
        two = np.zeros((len(lefts), d * d, d * d), np.complex128)
        h = 0
        for p, i in enumerate(lefts):
            if int(i) in special:
                two[p] = special[int(i)]
            else:
                two[p] = haar[h]
                h += 1
        circ.layers.append(Layer(one, lefts, two))
    return circ


WORKLOADS = {
    "brickwork_10q_d10_full": dict(nqudits=10, depth=10, d=2, maxsvals=None),
    "brickwork_48q_d24_chi128": dict(nqudits=48, depth=24, d=2, maxsvals=128),
    "brickwork_64q_d40_chi256": dict(nqudits=64, depth=40, d=2, maxsvals=256),
}


def workload(name: str, seed: int = 0, instance: int = 0) -> BrickworkCircuit:
    return brickwork(seed=seed, instance=instance, **WORKLOADS[name])


def _brickwork_args(args):
    return brickwork(*args[0], **args[1])


def build_many(specs, workers: Optional[int] = None) -> List[BrickworkCircuit]:
    """brickwork(*args, **kwargs) for every (args, kwargs) in ``specs``, spread
    over the host cores (a spawn-context process pool: safe in a process
    that already uses CUDA).  Drawing every gate from its own RandomState is
    the cost (~0.15 ms a gate; ~160k gates in the 512-circuit batch)."""
    import os
    specs = list(specs)
    workers = workers or min(len(specs), os.cpu_count() or 1, 32)
    if workers <= 1 or len(specs) < 8:
        return [_brickwork_args(s) for s in specs]
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_brickwork_args, specs, chunksize=max(1, len(specs) // (4 * workers))))


def mixed_batch(ncircuits: int = 512, seed: int = 0, workers: Optional[int] = None
                ) -> List[BrickworkCircuit]:
    """512 independent circuits: qubits U[16,48], depth U[8,32],
    maxsvals from {16,32,64,128}, 20% of two-qubit slots CNOT or CZ."""
    specs = []
    for k in range(ncircuits):
        rng = np.random.default_rng(np.random.SeedSequence([seed, k, 104729]))
        nq = int(rng.integers(16, 49))
        depth = int(rng.integers(8, 33))
        chi = int(rng.choice([16, 32, 64, 128]))
        specs.append(((nq, depth, 2, chi, seed, k), {"special_fraction": 0.2}))
    return build_many(specs, workers)


def qutrit_batch(ncircuits: int = 128, seed: int = 0, workers: Optional[int] = None
                 ) -> List[BrickworkCircuit]:
    """128 circuits of 32 qutrits, depth 30, maxsvals=192 (theta <= 576x576)."""
    return build_many([((32, 30, 3, 192, seed, k), {}) for k in range(ncircuits)], workers)


def gate_shapes(circ: BrickworkCircuit):
    """(one-qudit, two-qudit) Counters of (chi_l, chi_r) and (chi_l, chi_m,
    chi_r) over the circuit's gates.  The kept count of every two-qudit gate
    is min(maxsvals, min(chi_l d, d chi_r)), so the whole shape plan follows
    from the circuit without simulating it."""
    from collections import Counter
    n, d = circ.nqudits, circ.d
    bonds = [1] * (n + 1)
    two, one = Counter(), Counter()
    for lay in circ.layers:
        for i in range(n):
            one[(bonds[i], bonds[i + 1])] += 1
        for i in lay.pair_left:
            i = int(i)
            cl, cm, cr = bonds[i], bonds[i + 1], bonds[i + 2]
            two[(cl, cm, cr)] += 1
            r = min(cl * d, d * cr)
            bonds[i + 1] = r if circ.maxsvals is None else min(int(circ.maxsvals), r)
    return one, two


def estimated_cost(circ: BrickworkCircuit) -> float:
    """Relative device cost of a circuit: per two-qudit gate, the Jacobi SVD's
    L C^2 (L = max(m, n) rows, C = min(m, n) columns of the merged matrix) plus
    the merge's m n chi_m."""
    d = circ.d
    _, two = gate_shapes(circ)
    total = 0.0
    for (cl, cm, cr), count in two.items():
        m, n = cl * d, d * cr
        total += count * (max(m, n) * min(m, n) ** 2 + m * n * cm)
    return total


def shard_by_cost(circuits: Sequence[BrickworkCircuit], world: int) -> List[List[int]]:
    """Indices of ``circuits`` for each of ``world`` ranks: longest estimated
    cost first, each to the rank with the least work so far (every circuit
    exactly once; ranks may be empty when there are fewer circuits)."""
    if world < 1:
        raise ValueError("world must be at least 1")
    costs = [estimated_cost(c) for c in circuits]
    order = sorted(range(len(circuits)), key=lambda i: (-costs[i], i))
    loads = [0.0] * world
    shards = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (loads[q], q))
        shards[r].append(i)
        loads[r] += costs[i]
    return [sorted(s) for s in shards]


def sample_bitstrings(nqudits: int, d: int, count: int = 4096, seed: int = 0) -> np.ndarray:
    """Seeded computational-basis bitstrings for amplitude checks."""
    return np.random.default_rng(seed).integers(0, d, (count, nqudits))
