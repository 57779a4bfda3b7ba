"""Benchmark: two-qudit gates/s on the 64-qubit, depth-40, maxsvals=256 brickwork
circuit (theta up to 512x512 per gate), one JSON line on rank 0.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full circuit from |0...0>: 40 layers of seeded Haar one-qubit
gates on all 64 sites and Haar two-qubit gates on alternating pairs
(1260 two-qubit gates), then the state's norm.  ``value`` runs with the gates
already in HBM (``MPS.apply_layer_resident``); ``e2e`` runs the same circuit
through the public API with the gates in pinned host memory (``MPS.apply_layer``
copies them in every step) and reads the norm back.  Under torchrun each rank
simulates its own circuit instance on its own GPU (replicas; no collective in
the data path); the timed region is bracketed by a barrier and synchronize on
both sides and the slowest rank's time counts.

``--impl reference`` times the reference's CPU algorithm (the NumPy oracle
port: the same merge, LAPACK SVD and regauge per gate) on the host cores, on
a bounded sample of the same workload: one gate of every distinct gate shape
of the circuit, weighted by how often the shape occurs.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOAD = "brickwork_64q_d40_chi256"
METRIC = "chi=256 two-qudit gates/s (64q brickwork depth 40, maxsvals=256)"
UNIT = "two-qudit gates/s"


def gate_flops(m, n, chim, d):
    """Algorithmic flops of one two-qudit gate: merge, gate, complex thin SVD
    (4 x the Golub-Reinsch count 14 M N^2 + 8 N^3)."""
    big, small = max(m, n), min(m, n)
    return 8.0 * m * n * chim + 8.0 * m * n * d * d + 4.0 * (14.0 * big * small ** 2 + 8.0 * small ** 3)


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of a chi=256
# two-qudit call of 32 jobs, from one ncu capture per kernel (three launches
# each, caches left warm) scaled by the launch counts of one call: per sweep
# of the plain sweep kernel, and for the rest of the call (merge, LQ,
# post-GEMMs, sorts).  A call's traffic is sweeps x the first + the second.
SWEEP_TRAFFIC_BYTES = 1.12e9
CALL_OTHER_TRAFFIC_BYTES = 1.16e9


def replica_instance(rank: int) -> int:
    """Circuit instance simulated by a rank (replicas: one per GPU)."""
    return rank


def whole_job_rate(gates_per_step: int, steps: int, world: int, max_ms: float) -> float:
    """Gates of all ranks over the slowest rank's time."""
    return world * gates_per_step * steps / (max_ms / 1000.0)


def load_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def circuit_shapes(circ):
    """Counts of (chi_l, chi_r) over the circuit's one-qudit gates and of
    (chi_l, chi_m, chi_r) over its two-qudit gates (the deterministic shape
    plan of mpsim_gb300.circuits.gate_shapes)."""
    from mpsim_gb300.circuits import gate_shapes
    return gate_shapes(circ)


def _time_call(fn, min_seconds=0.02):
    reps, t0 = 0, time.perf_counter()
    while True:
        fn()
        reps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            return dt / reps


def cpu_sample(circ, seed=123, budget=12.0):
    """Cross-check of the reference arm: the NumPy oracle port (merge, LAPACK
    SVD, regauge; one-qudit contraction) timed on one gate of every distinct
    shape of ``circ``, weighted by how often each shape occurs, without the
    reference's per-gate norm sweep.  Returns two-qudit gates/s over the whole
    circuit and the seconds spent."""
    from oracle.ref_mps import OracleMPS
    from mpsim_gb300.circuits import haar_random_matrix
    rng = np.random.default_rng(seed)
    d = circ.d
    one, two = circuit_shapes(circ)
    t_start = time.perf_counter()

    def rnd(shape):
        t = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)
        return t / np.sqrt(t.size)

    calls = []                                   # (count, fn)
    g2 = haar_random_matrix(2, d, 1000)
    for (cl, cm, cr), count in two.items():
        a, b = rnd((cl, d, cm)), rnd((cm, d, cr))
        o = OracleMPS(2, d, np.complex64)

        def gate(o=o, a=a, b=b):
            o.sites = [a, b]
            o.apply_two_qudit_gate(g2, 0, 1, maxsvals=circ.maxsvals)
        calls.append((count, gate))
    g1 = haar_random_matrix(1, d, 1001)
    for (cl, cr), count in one.items():
        o = OracleMPS(2, d, np.complex64)
        s = rnd((cl, d, cr))

        def gate1(o=o, s=s):
            o.sites[0] = s
            o.apply_one_qudit_gate(g1, 0)
        calls.append((count, gate1))
    est = [count * _time_call(fn, 0.005) for count, fn in calls]
    spent = time.perf_counter() - t_start
    left = max(budget - spent, 0.0)
    total = 0.0
    for (count, fn), e in zip(calls, est):
        total += count * _time_call(fn, max(0.005, left * e / sum(est)))
    return sum(two.values()) / total, time.perf_counter() - t_start


REF_DIR = os.path.join(HERE, "baseline", "_ref")
SHIM_DIR = os.path.join(HERE, "oracle", "tn_shim")


def import_reference():
    """The reference's own package (pip-installed, unmodified, into
    baseline/_ref) over oracle/tn_shim -- a restatement of the TensorNetwork
    0.2.1 subset it calls, which is not installed anywhere -- with the two
    NumPy-2 patches it needs to import (``np.complex``, the ``newshape=``
    keyword of ``np.reshape``).  Returns ((tensornetwork, mpsim.core), None)
    or (None, reason)."""
    if not os.path.isfile(os.path.join(REF_DIR, "mpsim", "core.py")):
        return None, "baseline/_ref/mpsim is not installed"
    for p in (SHIM_DIR, REF_DIR):
        if p not in sys.path:
            sys.path.insert(0, p)
    if not hasattr(np, "complex"):
        np.complex = complex
    if not getattr(np.reshape, "_newshape_patch", False):
        orig = np.reshape

        def reshape(a, *args, **kw):
            if "newshape" in kw:
                kw["shape"] = kw.pop("newshape")
            return orig(a, *args, **kw)
        reshape._newshape_patch = True
        np.reshape = reshape
    try:
        import tensornetwork as tn
        import mpsim.core as core
    except Exception as exc:          # pragma: no cover - depends on the host
        return None, f"reference import failed: {exc!r}"
    if not os.path.realpath(core.__file__).startswith(os.path.realpath(REF_DIR)):
        return None, f"mpsim.core resolved to {core.__file__}, not baseline/_ref"
    return (tn, core), None


class ReferenceCircuit:
    """One seeded circuit driven through the reference's own public API:
    ``MPS.apply_one_qudit_gate`` / ``apply_two_qudit_gate(..., maxsvals=)``
    with complex64 gates (mpsim/core.py:753-845, 950-1161).  ``as_shipped``
    keeps the norm sweep the reference runs after every two-qudit gate
    (``self._norms.append(self.norm())``, core.py:1160-1161); otherwise
    ``MPS.norm`` is replaced by a constant for the duration of the layer."""

    def __init__(self, circ, tn, core):
        self.circ, self.tn, self.core = circ, tn, core
        self.mps = core.MPS(circ.nqudits, circ.d)
        self.next_layer = 0
        self.steady_from = None

    def run_layer(self, li, as_shipped=True):
        circ, tn, mps = self.circ, self.tn, self.mps
        lay = circ.layers[li]
        d = circ.d
        cls = type(mps)
        orig_norm = cls.norm
        if not as_shipped:
            cls.norm = lambda self: 0.0
        try:
            t0 = time.perf_counter()
            for i in range(circ.nqudits):
                mps.apply_one_qudit_gate(tn.Node(lay.one_q[i].astype(np.complex64)), i)
            for p, i in enumerate(lay.pair_left):
                g = lay.two_q[p].astype(np.complex64).reshape((d,) * 4)
                mps.apply_two_qudit_gate(tn.Node(g), int(i), int(i) + 1, maxsvals=circ.maxsvals)
            return time.perf_counter() - t0, len(lay.pair_left)
        finally:
            cls.norm = orig_norm

    def warm_to_steady(self):
        """Runs (as shipped) the layers up to and including the first one whose
        bonds are all at their final maximum; returns (seconds, two-qudit gates)."""
        t = g = 0
        final = max(C_gate_bonds(self.circ))
        while self.next_layer < len(self.circ.layers):
            dt, ng = self.run_layer(self.next_layer)
            t += dt
            g += ng
            self.next_layer += 1
            if max(self.mps.bond_dimensions()) >= final:
                break
        self.steady_from = self.next_layer
        return t, g

    def steady_layer(self, as_shipped=True):
        """The next steady-state layer (wrapping around to the first steady layer
        once the circuit ends: the bond dimensions stay at their maximum)."""
        if self.next_layer >= len(self.circ.layers):
            self.next_layer = self.steady_from
        dt, ng = self.run_layer(self.next_layer, as_shipped)
        self.next_layer += 1
        return dt, ng


def C_gate_bonds(circ):
    from mpsim_gb300.circuits import gate_shapes
    _, two = gate_shapes(circ)
    return [max(k[0], k[2]) for k in two]


def reference_rate(circ, steady_layers=1):
    """CPU baseline of the reference itself: the circuit's first layers through
    the first steady-state layer (timed), then ``steady_layers`` steady-state
    layers as shipped and one with the per-gate norm disabled.  The whole-circuit
    rate is extrapolated from the measured early part plus the steady-state rate
    for the remaining gates.  Returns a dict, or None with a reason."""
    ref, why = import_reference()
    if ref is None:
        return None, why
    tn, core = ref
    rc = ReferenceCircuit(circ, tn, core)
    t0 = time.perf_counter()
    t_early, g_early = rc.warm_to_steady()
    ts = gs = 0
    for _ in range(steady_layers):
        dt, ng = rc.steady_layer(True)
        ts += dt
        gs += ng
    dn, gn = rc.steady_layer(False)
    ngates = circ.n_two_qudit_gates
    rate = gs / ts
    whole = ngates / (t_early + (ngates - g_early) / rate)
    return {"whole": whole, "steady": rate, "steady_no_norms": gn / dn,
            "early_s": t_early, "early_gates": g_early, "spent": time.perf_counter() - t0}, None


def _blas_threads():
    try:
        from threadpoolctl import threadpool_info
        return sum(int(i.get("num_threads", 0)) for i in threadpool_info()
                   if i.get("user_api") == "blas") or None
    except Exception:
        return None


def run_reference(args, rank, world):
    """``--impl reference``: the reference's own MPS (baseline/_ref, unmodified,
    over oracle/tn_shim) on the host cores, rank 0 only.  Setup (untimed): the
    circuit's layers up to the first steady-state layer.  Warm-up steps: one
    steady-state layer each with the per-gate norm sweep disabled (the second
    variant).  Timed steps: one steady-state layer each as shipped.  ``value``
    = the whole circuit's two-qudit gates over the measured early layers plus
    the remaining gates at the timed steady-state rate."""
    if rank != 0:
        return 0
    from mpsim_gb300 import circuits as C
    name = args.workload if args.workload in C.WORKLOADS else WORKLOAD
    circ = C.workload(name)
    ref, why = import_reference()
    if ref is None:
        print(json.dumps({"impl": "reference", "unavailable": why}), flush=True)
        return 0
    tn, core = ref
    rc = ReferenceCircuit(circ, tn, core)
    t_early, g_early = rc.warm_to_steady()
    nn_t = nn_g = 0
    for _ in range(max(args.warmup, 1)):
        dt, ng = rc.steady_layer(as_shipped=False)
        nn_t += dt
        nn_g += ng
    ts = gs = 0
    t_all = time.perf_counter()
    for _ in range(args.steps):
        dt, ng = rc.steady_layer(as_shipped=True)
        ts += dt
        gs += ng
    total = time.perf_counter() - t_all
    steady = gs / ts
    ngates = circ.n_two_qudit_gates
    value = ngates / (t_early + (ngates - g_early) / steady)
    port, port_s = cpu_sample(circ, budget=3.0)
    cores = os.cpu_count()
    sample = (f"the reference's own mpsim.core (baseline/_ref, unmodified; TensorNetwork 0.2.1 "
              f"restated in oracle/tn_shim) on {circ.nqudits}-qubit depth-{circ.depth} "
              f"maxsvals={circ.maxsvals}: layers 0-{rc.steady_from - 1} timed once "
              f"({g_early} gates, {t_early:.1f}s), then {args.steps} steady-state layers as shipped "
              f"({gs} gates, {ts:.1f}s, per-gate norm sweep included); whole-circuit rate "
              f"extrapolated from both; {cores} host threads")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded Haar gates)",
        "config": {"workload": circ_name(circ), "sample": "steady-state layer per step",
                   "same_config": True},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "reference",
                         "sample": sample, "blas_threads": _blas_threads()},
        "variants": {"as_shipped_steady": steady,
                     "norms_disabled_steady": nn_g / nn_t if nn_t else None,
                     "oracle_port_cross_check": port},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def circ_name(circ):
    return f"brickwork_{circ.nqudits}q_d{circ.depth}_chi{circ.maxsvals}"


def batch_cpu_baseline(circs, states, budget_s=25.0):
    """The complex128 oracle (the FP64 restatement of the reference's path) on
    the cheapest circuits of the batch, as many as fit in ``budget_s``: its
    rate (the CPU baseline of the batched form) and, per circuit, the
    infidelity and norm error of the GPU state against it (MPS overlaps in
    complex128).  ``states``: callables returning circuit i's GPU state."""
    from oracle.ref_mps import OracleMPS, overlap_infidelity
    from mpsim_gb300.circuits import estimated_cost
    order = sorted(range(len(circs)), key=lambda i: estimated_cost(circs[i]))

    def oracle(c, dtype):
        o = OracleMPS(c.nqudits, c.d, dtype)
        kw = {} if c.maxsvals is None else {"maxsvals": c.maxsvals}
        for lay in c.layers:
            for q in range(c.nqudits):
                o.apply_one_qudit_gate(lay.one_q[q], q)
            for p, j in enumerate(lay.pair_left):
                o.apply_two_qudit_gate(lay.two_q[p], int(j), int(j) + 1, **kw)
        return o

    t0 = time.perf_counter()
    t_c128, gates, errs = 0.0, 0, []
    for i in order:
        c = circs[i]
        ta = time.perf_counter()
        o = oracle(c, np.complex128)
        t_c128 += time.perf_counter() - ta
        gates += c.n_two_qudit_gates
        o64 = oracle(c, np.complex64)
        g = OracleMPS(c.nqudits, c.d, np.complex128)
        g.sites = [t.detach().cpu().numpy().astype(np.complex128) for t in states(i).sites]
        on, gn = o.norm(), g.norm()
        errs.append({"circuit": i, "nqudits": c.nqudits, "depth": c.depth, "maxsvals": c.maxsvals,
                     "infidelity": overlap_infidelity(o, g),
                     "oracle_c64_infidelity": overlap_infidelity(o, o64),
                     "norm_rel_err": abs(gn - on) / max(on, 1e-300)})
        if time.perf_counter() - t0 > budget_s:
            break
    return gates / t_c128, t_c128, errs


def run_batch_workload(args, rank, world):
    """Multi-circuit workloads: batch_512_mixed and qutrit_128x32_d30_chi192.
    A step is every circuit of the batch from |0...0> to its last layer, run
    as one CircuitPlan (all circuits advance together, one call per layer and
    slot class) replayed as one CUDA graph.  With several ranks the batch is
    sharded by estimated cost (circuits.shard_by_cost: circuits are
    independent, no collective on the data path) and the step time is the
    slowest rank's: strong scaling."""
    import torch
    import __graft_entry__ as ge
    from mpsim_gb300 import circuits as C
    from mpsim_gb300 import _native
    from mpsim_gb300.plan import CircuitPlan

    ge.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    if args.workload == "batch_512_mixed":
        every = C.mixed_batch(args.ncircuits or 512, seed=0)
    else:
        every = C.qutrit_batch(args.ncircuits or 128, seed=0)
    mine = C.shard_by_cost(every, world)[rank]
    circs = [every[i] for i in mine]
    ngates_all = sum(c.n_two_qudit_gates for c in every)
    lib = _native.load()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def timed(fn):
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            flush.fill_(1)
            fn()
        e1.record()
        barrier()
        return max_over_ranks(e0.elapsed_time(e1))

    t_plan = time.perf_counter()
    plan = CircuitPlan(circs, device=dev, precision=args.precision) if circs else None
    plan_build_s = time.perf_counter() - t_plan
    states = [plan.state(i) for i in range(len(circs))] if plan else []

    def norms():
        return [s.norm() for s in states]

    for _ in range(max(args.warmup, 1)):
        if plan:
            plan.run()
    eager_ms = timed(lambda: (plan.run(), norms()) if plan else None)
    if plan:
        plan.capture()
        for _ in range(2):
            plan.replay(check=False)
    clocks = Clocks(local)
    clocks.start()
    l0 = lib.mps_kernel_launches()
    graph_ms = timed(lambda: (plan.replay(check=False), norms()) if plan else None)
    clk = clocks.stop()
    if plan:
        plan.check_status()
    # end to end through the public API: the plan built from the host
    # circuits (gates and job tables copied in), run, norms read back
    h2d = (plan.g1.numel() * 8 + plan.g2.numel() * 8 + plan.t1.numel() + plan.t2.numel()) if plan else 0
    barrier()
    w0 = time.perf_counter()
    e2e_norms = []
    for _ in range(args.steps):
        if circs:
            p2 = CircuitPlan(circs, device=dev, precision=args.precision)
            p2.run()
            e2e_norms = [p2.state(i).norm() for i in range(len(circs))]
            del p2
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - w0) * 1000.0)
    if rank == 0:
        peaks, peak_kind = load_peaks()
        peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
        flops = 0.0
        for c in every:
            for (cl, cm, cr), count in C.gate_shapes(c)[1].items():
                flops += count * gate_flops(cl * c.d, c.d * cr, cm, c.d)
        achieved = flops * args.steps / (graph_ms / 1000.0) / 1e12
        line = {
            "metric": f"two-qudit gates/s ({args.workload})",
            "value": ngates_all * args.steps / (graph_ms / 1000.0),
            "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": graph_ms / args.steps, "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded Haar gates)",
            "config": {"workload": args.workload, "circuits": len(every),
                       "two_qudit_gates_per_step": ngates_all,
                       "precision": args.precision,
                       "parallelism": f"cost-sharded x{world}",
                       "form": "CircuitPlan replayed as one CUDA graph",
                       "l2": "256 MiB buffer written at the start of every step"},
            "circuits_per_s": len(every) * args.steps / (graph_ms / 1000.0),
            "plan": {"value": ngates_all * args.steps / (eager_ms / 1000.0), "unit": UNIT,
                     "call": "CircuitPlan.run per step (eager), norms read back",
                     "build_s": plan_build_s},
            "e2e": {"value": ngates_all * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 8 * len(every),
                    "call": "CircuitPlan built from host circuits + run + norms, every step"},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "whole step (all launches), algorithmic flops of every gate",
                         "peak_source": f"bf16 sustained ({peak_kind})"},
            "gpu_launches": int(lib.mps_kernel_launches() - l0), "clocks": clk,
            "mean_norm": float(np.mean(norms())) if states else None,
        }
        if world == 1 and not args.no_cpu_baseline and circs:
            rate, dt, errs = batch_cpu_baseline(circs, lambda i: states[i])
            inf = [e["infidelity"] for e in errs]
            line["cpu_baseline"] = {
                "value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                "sample": f"complex128 NumPy oracle on the {len(errs)} cheapest circuits "
                          f"({dt:.1f}s)"}
            inf64 = [e["oracle_c64_infidelity"] for e in errs]
            line["error_vs_fp64_oracle"] = {
                "circuits": len(errs), "max_infidelity": max(inf),
                "median_infidelity": float(np.median(inf)),
                "max_norm_rel_err": max(e["norm_rel_err"] for e in errs),
                "oracle_c64_max_infidelity": max(inf64),
                "oracle_c64_median_infidelity": float(np.median(inf64)),
                "note": "the complex64 oracle's own infidelity against complex128 on the same "
                        "circuits: what truncated chaotic dynamics does to any complex64 run",
                "worst_circuits": sorted(errs, key=lambda e: -e["infidelity"])[:10]}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def batched_chi256(dev, njobs=512, reps=2, check=4):
    """The metric's own comparison: chi=256 two-qubit gates (theta 512 x 512,
    maxsvals=256) batched njobs to a call, through mps_apply_2q_batch in the
    plain form and in the mixed (tensor-core) form; gates/s of each, their
    ratio, and the mixed form's accuracy against complex128 LAPACK on `check`
    of the jobs: the truncated two-site block's infidelity, the largest
    relative error of the kept singular values (above 1e-3 s_0) and the
    truncation-weight error.  Synthetic sites: seeded complex Gaussians
    (left site scaled by 1/chi), seeded Haar gates; L2 flushed before each
    timed call."""
    import ctypes
    import torch
    from mpsim_gb300 import _native
    from mpsim_gb300.circuits import haar_random_matrix

    lib = _native.load()
    d, chi = 2, 256
    m = n = chi * d
    k = chi
    gen = torch.Generator(device=dev).manual_seed(2024)

    def sites(scale):
        t = torch.randn((njobs, chi, d, chi), dtype=torch.complex64, device=dev, generator=gen)
        return t * scale
    A, B = sites(1.0 / chi), sites(1.0)
    G = torch.from_numpy(np.stack([haar_random_matrix(2, d, 500 + q) for q in range(njobs)])
                         .astype(np.complex64)).to(dev)
    Ao = torch.empty((njobs, chi, d, k), dtype=torch.complex64, device=dev)
    Bo = torch.empty((njobs, k, d, chi), dtype=torch.complex64, device=dev)
    S = torch.zeros((njobs, min(m, n)), dtype=torch.float32, device=dev)   # every singular value
    disc = torch.zeros(njobs, dtype=torch.float64, device=dev)
    table = np.zeros(njobs, dtype=_native.JOB_DTYPE)
    for q in range(njobs):
        r = table[q]
        r["a"], r["b"], r["gate"] = A[q].data_ptr(), B[q].data_ptr(), G[q].data_ptr()
        r["a_out"], r["b_out"] = Ao[q].data_ptr(), Bo[q].data_ptr()
        r["svals"], r["discarded"] = S[q].data_ptr(), disc[q].data_ptr()
        r["chi_l"], r["chi_m"], r["chi_r"], r["k"], r["keep_left_canonical"] = chi, chi, chi, k, 1
    jobs = torch.from_numpy(table.view(np.uint8)).to(dev)
    nbytes = lib.mps_2q_workspace_bytes_mixed(njobs, m, n, d)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    out = {"config": f"{njobs} gates of theta {m} x {n}, maxsvals {k}, one call", "unit": UNIT}
    for prec in ("plain", "mixed"):
        p = _native.SvdParams()
        p.precision = _native.PRECISION_MIXED if prec == "mixed" else _native.PRECISION_PLAIN

        def call():
            _native.check(lib.mps_apply_2q_batch(stream, ctypes.c_void_p(jobs.data_ptr()), njobs,
                                                 m, n, d, ctypes.c_void_p(ws.data_ptr()), nbytes,
                                                 ctypes.byref(p)))
        call()
        times = []
        for _ in range(reps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            call()
            e1.record()
            torch.cuda.synchronize(dev)
            times.append(e0.elapsed_time(e1))
        out[prec] = {"value": njobs / (float(np.median(times)) / 1000.0), "ms_per_call": float(np.median(times)),
                     "sweeps": int(p.sweeps_out)}
    out["mixed_over_plain"] = out["mixed"]["value"] / out["plain"]["value"]
    # the mixed form's outputs (the last call) against complex128 LAPACK
    infid, sv_err, w_err = [], [], []
    for q in range(min(check, njobs)):
        a = A[q].cpu().numpy().astype(np.complex128)
        b = B[q].cpu().numpy().astype(np.complex128)
        g = G[q].cpu().numpy().astype(np.complex128).reshape(d, d, d, d)
        mm = (a.reshape(m, chi) @ b.reshape(chi, n)).reshape(chi, d, d, chi)
        th = np.einsum("xyab,labr->lxyr", g, mm).reshape(m, n)
        u, sv, vh = np.linalg.svd(th, full_matrices=False)
        best = (u[:, :k] * sv[:k]) @ vh[:k]
        got = Ao[q].cpu().numpy().astype(np.complex128).reshape(m, k) @ \
            Bo[q].cpu().numpy().astype(np.complex128).reshape(k, n)
        ov = abs(np.vdot(best, got)) ** 2 / (np.vdot(best, best).real * np.vdot(got, got).real)
        infid.append(1.0 - ov)
        s_gpu = S[q].cpu().numpy().astype(np.float64)[:k]
        keep = sv[:k] > 1e-3 * sv[0]
        sv_err.append(float(np.max(np.abs(s_gpu[keep] - sv[:k][keep]) / sv[:k][keep])))
        wt = float(np.sum(sv[k:] ** 2))
        w_err.append(abs(float(disc[q].item()) - wt) / max(wt, 1e-300))
    out["mixed_accuracy_vs_fp64"] = {"jobs_checked": len(infid), "max_infidelity": max(infid),
                                     "max_sv_rel_error": max(sv_err),
                                     "max_truncation_weight_rel_error": max(w_err)}
    del A, B, G, Ao, Bo, ws, flush
    torch.cuda.empty_cache()
    return out


def run_case(args):
    """Single-purpose chi=256 workloads for timing and profiling one kernel
    family (``--case``), each run ``--steps`` times after ``--warmup`` runs,
    timed with CUDA events on the launching stream after a 256 MiB buffer is
    written (so L2 holds none of the case's data); one JSON line.

      layer256        one mps_apply_2q_batch call: 32 jobs of theta 512 x 512
                      (random sites, Haar gates), plain form
      layer256_mixed  the same call in MPS_PRECISION_MIXED
      batched256      the same with 512 jobs (the batched form), plain
      batched256_mixed  ... and in MPS_PRECISION_MIXED
      onequbit256     one mps_apply_1q_batch over 64 sites of (256, 2, 256):
                      HBM-bound, 2 x 64 x 1 MiB moved
      norm256         MPS.norm of a 64-site chi=256 state (the overlap sweep)
      tcgemm          mps_cgemm_tc, 1024 x 1024 x 1024 complex
    """
    import ctypes
    import torch
    import __graft_entry__ as ge
    from mpsim_gb300 import _native
    from mpsim_gb300.circuits import haar_random_matrix
    from mpsim_gb300.core import MPS

    ge.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lib = _native.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(0)
    d, chi = 2, 256

    def rand_sites(n, cl, cr, scale):
        t = rng.normal(size=(n, cl, d, cr)) + 1j * rng.normal(size=(n, cl, d, cr))
        return torch.from_numpy((t * scale).astype(np.complex64)).to(dev)

    keep = []
    if args.case in ("layer256", "layer256_mixed", "batched256", "batched256_mixed"):
        njobs = 512 if args.case.startswith("batched") else 32
        A, B = rand_sites(njobs, chi, chi, 1.0 / chi), rand_sites(njobs, chi, chi, 1.0)
        G = torch.from_numpy(np.stack([haar_random_matrix(2, d, 100 + q) for q in range(njobs)])
                             .astype(np.complex64)).to(dev)
        Ao = torch.empty((njobs, chi, d, chi), dtype=torch.complex64, device=dev)
        Bo = torch.empty_like(Ao)
        table = np.zeros(njobs, dtype=_native.JOB_DTYPE)
        for q in range(njobs):
            r = table[q]
            r["a"], r["b"], r["gate"] = A[q].data_ptr(), B[q].data_ptr(), G[q].data_ptr()
            r["a_out"], r["b_out"] = Ao[q].data_ptr(), Bo[q].data_ptr()
            r["chi_l"], r["chi_m"], r["chi_r"], r["k"], r["keep_left_canonical"] = chi, chi, chi, chi, 1
        jobs = torch.from_numpy(table.view(np.uint8)).to(dev)
        nbytes = lib.mps_2q_workspace_bytes_mixed(njobs, 2 * chi, 2 * chi, d)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        params = _native.SvdParams()
        params.precision = (_native.PRECISION_MIXED if args.case.endswith("_mixed")
                            else _native.PRECISION_PLAIN)

        def once():
            _native.check(lib.mps_apply_2q_batch(stream, ctypes.c_void_p(jobs.data_ptr()), njobs,
                                                 2 * chi, 2 * chi, d, ctypes.c_void_p(ws.data_ptr()),
                                                 nbytes, ctypes.byref(params)))
        work = njobs * gate_flops(2 * chi, 2 * chi, chi, d) / 1e12
        unit = "TFLOP/s (algorithmic, per call)"
    elif args.case == "onequbit256":
        nsite = 64
        S = rand_sites(nsite, chi, chi, 1.0)
        U = torch.from_numpy(np.stack([haar_random_matrix(1, d, q) for q in range(nsite)])
                             .astype(np.complex64)).to(dev)
        t1 = np.zeros(nsite, dtype=_native.JOB1_DTYPE)
        for q in range(nsite):
            t1[q]["site"], t1[q]["gate"] = S[q].data_ptr(), U[q].data_ptr()
            t1[q]["chi_l"], t1[q]["chi_r"] = chi, chi
        jt = torch.from_numpy(t1.view(np.uint8)).to(dev)

        def once():
            _native.check(lib.mps_apply_1q_batch(stream, ctypes.c_void_p(jt.data_ptr()), nsite, d))
        work = 2 * S.numel() * 8 / 1e9
        unit = "GB/s (site bytes read + written)"
    elif args.case == "norm256":
        n = 64
        sites = []
        for i in range(n):
            cl = 1 if i == 0 else chi
            cr = 1 if i == n - 1 else chi
            sites.append(rand_sites(1, cl, cr, 1.0 / np.sqrt(cl * d))[0])
        mps = MPS.from_sites(sites, d)

        def once():
            mps.norm()
        work = sum(8.0 * d * t.shape[0] * t.shape[2] * (t.shape[0] + t.shape[2])
                   for t in sites) / 1e12
        unit = "TFLOP/s (overlap sweep, algorithmic)"
    elif args.case == "tcgemm":
        m = n = k = 1024
        a, b = rand_sites(1, m, k // d, 1.0)[0], rand_sites(1, k, n // d, 1.0)[0]
        c = torch.empty((m, n), dtype=torch.complex64, device=dev)

        def once():
            _native.check(lib.mps_cgemm_tc(stream, m, n, k, ctypes.c_void_p(a.data_ptr()), k, 1, 0,
                                           ctypes.c_void_p(b.data_ptr()), n, 1, 0,
                                           ctypes.c_void_p(c.data_ptr()), n, 1, 0, 0, 0, 0))
        work = 8.0 * m * n * k / 1e12
        unit = "TFLOP/s (complex 4M count)"
    else:
        raise SystemExit(f"unknown case {args.case}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        once()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        flush.fill_(1)                   # L2 (126 MB) holds nothing of the case
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        once()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    peaks, kind = load_peaks()
    line = {"case": args.case, "ms_median": ms, "ms": times, "achieved": work / (ms / 1000.0),
            "unit": unit, "launches_total": int(lib.mps_kernel_launches())}
    if unit.startswith("GB/s"):
        line["frac_of_hbm_copy"] = line["achieved"] / peaks["hbm_gbs"]
        line["peak_source"] = f"hbm_gbs ({kind})"
    if args.case in ("layer256", "layer256_mixed", "batched256", "batched256_mixed"):
        line["sweeps"] = int(params.sweeps_out)
    if args.case.endswith("_mixed"):
        # cycles of the tensor-core visits per step (one more call, counters
        # reset before it): Gram, rotations on G, update; and the visit count
        cyc = (ctypes.c_ulonglong * 10)()
        _native.check(lib.mps_tc_profile(cyc, 1))
        once()
        torch.cuda.synchronize()
        _native.check(lib.mps_tc_profile(cyc, 1))
        nv = max(int(cyc[3]), 1)
        line["tc_visits"] = int(cyc[3])
        line["tc_visits_rotating"] = int(cyc[4])
        line["tc_rotating_steps_per_rotating_visit"] = cyc[5] / max(int(cyc[4]), 1)
        line["tc_pairs_per_rotating_step"] = cyc[6] / max(int(cyc[5]), 1)
        line["tc_wait_cycles_per_visit"] = cyc[7] / nv
        line["tc_ctas_per_sweep"] = cyc[9] / max(int(params.sweeps_out), 1)
        line["tc_cta_lifetime_cycles"] = cyc[8] / max(int(cyc[9]), 1)
        line["tc_cycles_per_visit"] = {"gram": cyc[0] / nv, "rotations": cyc[1] / nv,
                                       "update": cyc[2] / nv}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ncircuits", type=int, default=0)
    ap.add_argument("--precision", default="plain", choices=["plain", "mixed", "auto"])
    ap.add_argument("--case", default=None,
                    choices=["layer256", "layer256_mixed", "batched256", "batched256_mixed",
                             "onequbit256", "norm256", "tcgemm"],
                    help="time one kernel family on a chi=256 case (for profiling)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.case:
        return run_case(args)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload in ("batch_512_mixed", "qutrit_128x32_d30_chi192"):
        return run_batch_workload(args, rank, world)

    import torch
    import __graft_entry__ as ge
    from mpsim_gb300 import circuits as C
    from mpsim_gb300 import _native
    from mpsim_gb300.core import MPS, MPSOperation
    from mpsim_gb300.gates import Node

    ge.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    circ = C.workload(args.workload, seed=0, instance=replica_instance(rank))
    maxs = circ.maxsvals
    d = circ.d
    dev_layers = [(torch.from_numpy(l.one_q.astype(np.complex64)).to(dev), l.pair_left,
                   torch.from_numpy(l.two_q.astype(np.complex64)).to(dev)) for l in circ.layers]
    host_layers = []
    for l in circ.layers:
        one = torch.from_numpy(l.one_q.astype(np.complex64)).pin_memory()
        two = torch.from_numpy(l.two_q.astype(np.complex64)).pin_memory()
        host_layers.append((one.numpy(), l.pair_left, two.numpy()))
    h2d = sum(a.nbytes + c.nbytes for a, _, c in host_layers)
    ngates = circ.n_two_qudit_gates
    lib = _native.load()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step_resident(timing=None):
        flush.fill_(1)
        mps = MPS(circ.nqudits, d, precision=args.precision)
        mps.timing = timing
        for one, left, two in dev_layers:
            mps.apply_layer_resident(one, left, two, maxsvals=maxs)
        return mps.norm()

    def step_e2e():
        flush.fill_(1)
        mps = MPS(circ.nqudits, d, precision=args.precision)
        for one, left, two in host_layers:
            mps.apply_layer(one, left, two, maxsvals=maxs)
        return mps.norm()

    # the reference's own call: MPS.apply with a list of MPSOperation per layer
    host_ops = []
    for one, left, two in host_layers:
        ops = [MPSOperation(Node(one[i]), i) for i in range(circ.nqudits)]
        ops += [MPSOperation(Node(two[p].reshape((d,) * 4)), (int(i), int(i) + 1))
                for p, i in enumerate(left)]
        host_ops.append(ops)

    def step_apply_ops():
        flush.fill_(1)
        mps = MPS(circ.nqudits, d, precision=args.precision)
        for ops in host_ops:
            mps.apply(ops, maxsvals=maxs)
        return mps.norm()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    for _ in range(args.warmup):
        step_resident()
    clocks = Clocks(local)
    clocks.start()
    timing = []
    launches0 = lib.mps_kernel_launches()
    barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    norms = []
    for _ in range(args.steps):
        norms.append(step_resident(timing))
    ev1.record()
    barrier()
    launches = lib.mps_kernel_launches() - launches0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    ms = max_over_ranks(ms)
    value = whole_job_rate(ngates, args.steps, world, ms)

    # roofline of the batched two-qudit launch on chi=256 layers
    peaks, peak_kind = load_peaks()
    full = [(nj, sw, a.elapsed_time(b)) for (nj, mm, nn, sw, a, b) in timing
            if mm == 2 * 256 and nn == 2 * 256]
    f_gate = gate_flops(512, 512, 256, 2)
    if full:
        tot_fl = sum(nj * f_gate for nj, _, _ in full)
        tot_ms = sum(t for _, _, t in full)
        achieved = tot_fl / (tot_ms / 1000.0) / 1e12
        mean_sweeps = sum(sw for _, sw, _ in full) / len(full)
    else:
        achieved, mean_sweeps = None, None
    peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))

    # end to end through the public API, host buffers
    for _ in range(1):
        step_e2e()
    barrier()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step_e2e()
    e1.record()
    barrier()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1))
    e2e_value = whole_job_rate(ngates, args.steps, world, e2e_ms)

    step_apply_ops()
    barrier()
    a0 = torch.cuda.Event(enable_timing=True)
    a1 = torch.cuda.Event(enable_timing=True)
    a0.record()
    for _ in range(args.steps):
        step_apply_ops()
    a1.record()
    barrier()
    ops_ms = max_over_ranks(a0.elapsed_time(a1))
    ops_value = whole_job_rate(ngates, args.steps, world, ops_ms)

    # the same circuit planned once (CircuitPlan: every table and buffer made
    # before the first launch), run eagerly and replayed as one CUDA graph
    from mpsim_gb300.plan import CircuitPlan
    plan = CircuitPlan([circ], device=dev, precision=args.precision)
    plan_state = plan.state(0)

    def timed(fn):
        fn()
        barrier()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(args.steps):
            flush.fill_(1)
            fn()
            plan_state.norm()
        t1.record()
        barrier()
        return max_over_ranks(t0.elapsed_time(t1))

    plan_ms = timed(plan.run)
    plan_norm = plan_state.norm()
    plan.capture()
    graph_ms = timed(lambda: plan.replay(check=False))
    plan.check_status()
    graph_norm = plan_state.norm()

    batched = None
    if rank == 0 and world == 1 and args.workload == WORKLOAD:
        batched = batched_chi256(dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r, why = reference_rate(circ)
        if r is not None:
            cpu = {"value": r["whole"], "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                   "sample": (f"the reference's own mpsim.core over oracle/tn_shim: layers up to the "
                              f"first steady-state one ({r['early_gates']} gates, {r['early_s']:.1f}s), "
                              f"one steady-state layer as shipped and one with the per-gate norm "
                              f"disabled ({r['spent']:.1f}s in all); whole-circuit rate extrapolated"),
                   "steady": r["steady"], "steady_no_norms": r["steady_no_norms"]}
        else:
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                   "sample": f"unavailable: {why}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "synthetic (seeded Haar gates)",
            "config": {"workload": args.workload, "nqudits": circ.nqudits, "depth": circ.depth,
                       "maxsvals": maxs, "two_qudit_gates_per_step": ngates,
                       "precision": {"plain": "plain complex64, FP32 SIMT",
                                     "mixed": "mixed: tcgen05 split-bf16 block Jacobi for "
                                              "left-canonical gates of 64+ columns, FP32 SIMT "
                                              "elsewhere",
                                     "auto": "auto: per call, the form the tuning table "
                                             "measured faster"}[args.precision],
                       "parallelism": f"replicas x{world}",
                       "l2": "256 MiB buffer written at the start of every step"},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
                         "traffic": (mean_sweeps * SWEEP_TRAFFIC_BYTES + CALL_OTHER_TRAFFIC_BYTES
                                     if (args.workload == WORKLOAD and mean_sweeps
                                         and args.precision == "plain") else None),
                         "traffic_unit": "bytes per call (one chi=256 layer, 32 gates)",
                         "kernel": "mps_apply_2q_batch on chi=256 layers (merge + Jacobi SVD + "
                                   "regauge, all launches of one call)",
                         "flops_per_gate": f_gate, "peak_source": f"bf16 sustained ({peak_kind})",
                         "mean_sweeps": mean_sweeps,
                         "fp32_simt_nominal_frac": (achieved / 80.5) if achieved else None},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": 8, "call": "MPS.apply_layer per layer, pinned host gates"},
            "e2e_reference_api": {"value": ops_value, "unit": UNIT,
                                  "call": "MPS.apply([MPSOperation, ...], maxsvals=256) per layer, "
                                          "host gates, norm read back"},
            "plan": {"value": whole_job_rate(ngates, args.steps, world, plan_ms), "unit": UNIT,
                     "call": "CircuitPlan.run per step (all tables and buffers planned once), "
                             "norm read back", "final_norm": plan_norm},
            "graph": {"value": whole_job_rate(ngates, args.steps, world, graph_ms), "unit": UNIT,
                      "call": "CircuitPlan captured as one CUDA graph, replayed per step, norm "
                              "read back", "final_norm": graph_norm},
            "gpu_launches": int(launches),
            "clocks": clk,
            "final_norm": float(norms[-1]) if norms else None,
        }
        if batched is not None:
            line["batched_chi256"] = batched
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
