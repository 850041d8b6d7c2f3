"""The multi-GPU path is independent replicas (one run per rank, no data-path
collective); its host logic -- max-over-ranks timing and the whole-job value --
runs here as two gloo ranks on CPU."""
import os
import socket
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert bench.dist_env() == (ws, rank, rank)
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
    m = bench.max_over_ranks(ms, ws)
    bench.barrier(ws)
    out[rank] = (m, bench.whole_job_steps_per_s(m, 10, ws))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    m, v = out[0]
    assert m == 150.0
    assert abs(v - 2 * 10 / 0.150) < 1e-9
