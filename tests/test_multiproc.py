"""bench.py's N > 1 path runs independent replicas ("replicas only": the
operator does not shard across GPUs here) and aggregates them as
units of all ranks / max-over-ranks time.  Checked with world_size 2 on the
gloo backend, on CPU."""
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


def _worker(rank, ws, port, out):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = [12.0, 20.0][rank]
    value, t_max = bench.aggregate_replicas(ms, units_per_step=1_000_000, steps=10)
    out[rank] = (value, t_max)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_gloo_world_size_2():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        value, t_max = res[r]
        assert t_max == pytest.approx(20.0)
        # 2 ranks x 1e6 units x 10 steps in 20 ms = 1.0 G units/s
        assert value == pytest.approx(1.0)


def test_single_process_aggregation():
    import bench
    value, t_max = bench.aggregate_replicas(8.0, units_per_step=2_000_000, steps=4)
    assert t_max == 8.0 and value == pytest.approx(1.0)
