"""bench.py with --gpus N runs N independent replicas of the case (the path
needs a halo exchange only when one case is split, which this build does not
do); the whole-job value takes the slowest rank's time.  The aggregation runs
here as two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [10.0, 12.5][rank]
    value, ms_max = bench.replica_value(ms, 64, world, "cpu")
    q.put((rank, value, ms_max))
    dist.destroy_process_group()


def test_replica_value_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms in out:
        assert ms == 12.5
        assert value == pytest.approx(2 * 64 ** 3 / 12.5e-3 / 1e6)
