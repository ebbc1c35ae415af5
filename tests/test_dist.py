"""The multi-rank path of bench.py on CPU: two gloo ranks (world size 2,
rendezvous on 127.0.0.1) check the point sharding (each rank its own fixed
share, no exchange) and the max-over-ranks timing that sets the job's
throughput."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, outdir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, rk, _ = bench._dist_env()
    pts = bench.rank_points(rk, m=64)
    times = bench.max_over_ranks([1.0 + rk, 10.0 - rk, 0.5 * (rk + 1)], dist)
    rate = bench.job_rate(1000.0, 4, ws, times[0])
    dist.barrier()
    np.savez(os.path.join(outdir, f"rank{rk}.npz"), pts=pts, times=np.array(times), rate=rate, ws=ws)
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    r0, r1 = (np.load(tmp_path / f"rank{r}.npz") for r in range(2))
    # each rank evaluates its own share: same shape, different points, rank 0 = the workload's own points
    assert r0["pts"].shape == r1["pts"].shape == (64, 16)
    assert not np.allclose(r0["pts"], r1["pts"])
    sys.path.insert(0, ROOT)
    from numcosmo_gb300 import workloads as wl

    assert np.array_equal(r0["pts"], wl.config2().points[:64])
    # the slowest rank sets the job time, identically on every rank
    assert np.array_equal(r0["times"], [2.0, 10.0, 1.0]) and np.array_equal(r1["times"], r0["times"])
    assert float(r0["rate"]) == pytest.approx(2 * 1000.0 * 4 / 2.0) and int(r0["ws"]) == 2


def test_single_rank_helpers():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([3.0, 1.0]) == [3.0, 1.0]
    assert bench.job_rate(10.0, 2, 1, 4.0) == pytest.approx(5.0)
    a, b = bench.rank_points(1, m=8), bench.rank_points(1, m=8)
    assert np.array_equal(a, b)
