"""Replicas-only multi-GPU form, exercised with two gloo ranks on CPU.

The DEM step does not exchange anything between GPUs: `bench.py --gpus N`
runs one independent copy of the workload per rank and combines the ranks
only after the timed region (MAX of the times, sum of the work).  Here each
rank steps its own copy of a small sphere drop with the CPU oracle, and the
test checks that:
  * the replicas stay bit-identical (no rank depends on another rank),
  * bench.replica_totals takes the slowest rank's time and counts the work
    of every rank.
"""
import os
import socket
import sys
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WS = 2
STEPS = 3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(WS))
    dist.init_process_group("gloo", rank=rank, world_size=WS)
    try:
        import bench
        import kseq
        import pyoracle
        from xdynamics_dll_gb300 import scenes
        o = pyoracle.Oracle()
        o.set_threads(1)
        be = kseq.OracleBackend(o)
        sc = scenes.sphere_drop(n_per_layer_side=8, layers=2)
        s = kseq.state_arrays(sc, history=False)
        t0 = time.perf_counter()
        for _ in range(STEPS):
            kseq.sphere_step(be, sc, s, (), compat=0)
        secs = time.perf_counter() - t0
        # a deliberately slower rank 1, so MAX over ranks is observable
        secs_reported = secs * (1.0 if rank == 0 else 3.0)
        digest = torch.tensor(np.frombuffer(np.ascontiguousarray(s["pos"]).tobytes(), dtype=np.int64).copy())
        gathered = [torch.zeros_like(digest) for _ in range(WS)]
        dist.all_gather(gathered, digest)
        same = all(torch.equal(g, gathered[0]) for g in gathered)
        times = [torch.zeros(1, dtype=torch.float64) for _ in range(WS)]
        dist.all_gather(times, torch.tensor([secs_reported], dtype=torch.float64))
        value, value64, e2e, s64, sx = bench.replica_totals(secs_reported, secs_reported, secs_reported / sc.np_,
                                                            WS, sc.np_, STEPS, torch.device("cpu"))
        if rank == 0:
            out.put(dict(same=same, times=[float(t) for t in times], value=value, value64=value64, e2e=e2e,
                         sx=sx, n=sc.np_))
    finally:
        dist.destroy_process_group()


def test_two_replicas_are_independent_and_timed_by_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(WS)]
    for p in procs:
        p.start()
    try:
        res = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    assert res["same"], "replicas diverged: a rank depended on another"
    slow = max(res["times"])
    assert res["sx"] == pytest.approx(slow)
    assert res["value"] == pytest.approx(WS * res["n"] * STEPS / slow)
    assert res["value64"] == pytest.approx(WS * res["n"] * STEPS / slow)
    assert res["e2e"] == pytest.approx(WS * res["n"] / slow)
