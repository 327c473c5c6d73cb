"""The N>1 path of bench.py on the CPU with two gloo ranks.

Every rank renders its own replica (the path shards by pixel, sample and job
without any exchange step, so the multi-GPU mode is replicas); rank 0 reports
the samples of all ranks over the slowest rank's time.  Here each rank renders
a small frame with the CPU oracle, and the aggregation helpers of bench.py are
checked against the values the ranks report.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      OMP_NUM_THREADS="2")
    import time

    import torch.distributed as dist

    import bench
    import oracle
    from photon_gb300 import workloads
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, cam, st = workloads.feature_scene("basic", res=24)
    st.pixel_samples = 1 + rank
    r = oracle.CpuRenderer("oracle")
    r.set_scene(sc)
    bench.barrier(world)
    t = time.perf_counter()
    r.render(cam, st, True)
    dt = time.perf_counter() - t
    samples = st.width * st.height * st.pixel_samples
    tmax = bench.dist_max(dt, world)
    total = bench.dist_sum(samples, world)
    q.put((rank, dt, samples, tmax, total, float(r.read("color")[..., :3].mean())))
    dist.destroy_process_group()


def test_two_rank_replicas_aggregate(oracle_lib):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, dt0, s0, tmax0, tot0, m0), (r1, dt1, s1, tmax1, tot1, m1) = res
    assert tmax0 == tmax1 == max(dt0, dt1)
    assert tot0 == tot1 == s0 + s1
    assert m0 > 0 and m1 > 0
