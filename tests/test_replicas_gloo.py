"""The multi-process path of bench.py on CPU: world size 2 over gloo (127.0.0.1).  The render
shards as independent replicas (one process per GPU, no collective on the data path); what the
ranks share is the slowest replica's time, from which the whole-job throughput is computed, and
the reference arm's rule that rank 0 alone times the CPU baseline."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, seconds, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, dist = bench.dist_setup(world)
    assert dist is not None and dist.get_backend() == "gloo"
    slowest = bench.barrier_max(dist, seconds[rank])
    # the reference arm: every rank but 0 returns before doing any work
    ran = []
    bench.cpu_port_sample = lambda *a, **k: ran.append(1) or None
    if rank != 0:
        bench.run_reference(None, bench.WORKLOAD)
    out.put((r, w, slowest, bench.replica_throughput(w, 1000, slowest), len(ran)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_share_the_slowest_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    seconds = [0.25, 0.5]
    procs = [ctx.Process(target=_replica, args=(r, 2, port, seconds, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == pytest.approx(0.5) for r in res)           # max over ranks, on every rank
    assert all(r[3] == pytest.approx(2 * 1000 / 0.5) for r in res)  # whole job: 2 replicas' units
    assert res[1][4] == 0                                          # rank 1 did no reference work


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    r, w, local, dist = bench.dist_setup(1)
    assert (r, w, local, dist) == (0, 1, 0, None)
    assert bench.barrier_max(None, 3.5) == 3.5
    assert bench.replica_throughput(1, 1000, 0.5) == pytest.approx(2000)
