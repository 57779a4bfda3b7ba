"""The N>1 bench path on CPU: replicas, one circuit instance per rank, no
collective on the data path; only the slowest rank's time is reduced (MAX)
and the whole-job rate counts every rank's gates.  world_size 2, gloo."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import time
    import torch
    import torch.distributed as dist
    import bench
    from mpsim_gb300 import circuits as C
    from oracle.ref_mps import OracleMPS
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    circ = C.brickwork(6, 3, d=2, maxsvals=4, seed=0, instance=bench.replica_instance(rank))
    t0 = time.perf_counter()
    o = OracleMPS(circ.nqudits, circ.d, np.complex128)
    for kind, sites, mat in circ.operations():
        if kind == 1:
            o.apply_one_qudit_gate(mat, sites[0])
        else:
            o.apply_two_qudit_gate(mat, *sites, maxsvals=4)
    ms = (time.perf_counter() - t0) * 1000.0 + 50.0 * rank
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    rate = bench.whole_job_rate(circ.n_two_qudit_gates, 1, world, float(t.item()))
    out.put((rank, ms, float(t.item()), rate, circ.layers[0].two_q[0].tobytes(),
             circ.n_two_qudit_gates))
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, mx0, rate0, g0, n0), (r1, ms1, mx1, rate1, g1, n1) = res
    assert mx0 == mx1 == max(ms0, ms1)
    assert n0 == n1 == 8
    assert rate0 == rate1 == 2 * n0 / (mx0 / 1000.0)
    assert g0 != g1            # each rank simulates its own circuit instance


def _shard_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    from mpsim_gb300 import circuits as C
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    every = C.mixed_batch(64, seed=0)
    mine = C.shard_by_cost(every, world)[rank]
    cost = sum(C.estimated_cost(every[i]) for i in mine)
    t = torch.tensor([cost], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out.put((rank, mine, cost, float(t.item())))
    dist.destroy_process_group()


def test_batch_sharded_by_cost_over_gloo():
    """The multi-circuit bench path with two ranks: every circuit on exactly
    one rank, the ranks' estimated work within 10% of each other, and the
    slowest rank's figure reduced with MAX."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, m0, c0, x0), (_, m1, c1, x1) = res
    assert sorted(m0 + m1) == list(range(64))
    assert not set(m0) & set(m1)
    assert x0 == x1 == max(c0, c1)
    assert max(c0, c1) / min(c0, c1) < 1.10
