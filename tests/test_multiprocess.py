"""The N > 1 path of bench.py runs independent replicas ("replicas only"): whole-job
throughput = units summed over ranks / slowest rank's time.  Checked with world_size 2 on
CPU over gloo."""
import os
import socket
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    dist, r, ws, local = bench.dist_setup()
    units, seconds = 1000.0 * (rank + 1), 2.0 + rank  # rank 1 is slower
    value, tmax = bench.aggregate(dist, units, seconds)
    q.put((r, ws, value, tmax))
    dist.destroy_process_group()


def test_replica_aggregation_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    for r, ws, value, tmax in res:
        assert ws == 2 and tmax == 3.0
        assert abs(value - 3000.0 / 3.0) < 1e-9
