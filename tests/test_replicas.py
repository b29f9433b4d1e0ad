"""The replica driver on CPU with a world of two gloo ranks: barriers, the
maximum of the ranks' times and the whole-job rate (each rank runs the whole
workload; the job lasts as long as its slowest rank).  Each rank also drops
a cutter on a small mesh with the CPU oracle and the ranks compare results
(independent replicas agree exactly)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch
    from opencamlib_gb300 import replicas, workloads as w, cutters as cu
    from oracle import checker
    r, n, local, dist = replicas.setup("gloo")
    assert (r, n, local) == (rank, world, rank)
    replicas.barrier(dist)
    t = 0.25 + 0.5 * rank  # this rank's time for its units
    slowest = replicas.max_over_ranks(t, dist)
    rate = replicas.whole_job_rate(1000, n, slowest)
    tris = w.heightfield(10, 10, seed=3)
    z = checker.drop(tris, cu.BallCutter(6.0, 20.0), w.raster(8, 8, 12.0), "port", nthreads=1)[0]
    zs = [torch.zeros_like(torch.from_numpy(z)) for _ in range(n)]
    dist.all_gather(zs, torch.from_numpy(z))
    out[rank] = (slowest, rate, all(torch.equal(zs[0], q) for q in zs))
    replicas.barrier(dist)
    replicas.teardown(dist)


def test_two_gloo_replicas():
    from oracle import checker
    checker.build(ref=False)
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(k, 2, port, out)) for k in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for k in range(2):
        slowest, rate, same = res[k]
        assert slowest == pytest.approx(0.75)
        assert rate == pytest.approx(2 * 1000 / 0.75)
        assert same


def test_single_process_needs_no_group(monkeypatch):
    from opencamlib_gb300 import replicas
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    r, n, local, dist = replicas.setup("gloo")
    assert (r, n, local, dist) == (0, 1, 0, None)
    assert replicas.max_over_ranks(3.5, None) == 3.5
    assert replicas.whole_job_rate(10, 1, 2.0) == 5.0
    assert np.isfinite(replicas.whole_job_rate(1, 1, 1e-9))
