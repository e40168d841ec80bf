"""Host logic of the multi-GPU form (replicas only), on CPU with gloo.

bench.py runs one independent instance per rank; the only cross-rank work is
a barrier around the timed region and a max-reduction of the timings."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    d = bench.Dist()
    d.barrier()
    m = d.max(10.0 + rank)
    d.barrier()
    d.close()
    q.put((rank, m))


@pytest.mark.parametrize("world", [2])
def test_dist_max_over_ranks(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {r: 10.0 + world - 1 for r in range(world)}


def test_clock_summary_parsing():
    import bench

    lines = ["0, 1980, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
             "0, 2070, 2070, 1200.1, 0x4, Not Active, Not Active, Not Active, Active",
             "0, 2010, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    s = bench.summarize_clocks(lines)
    assert s["sm_mhz"] == 2010 and s["sm_max_mhz"] == 2070 and s["reasons"] == ["sw_power_cap"]
