"""The N > 1 bench path on CPU: two gloo ranks combine their replica timings (max over ranks) into
one whole-job throughput, as bench.py does over NCCL on GPUs."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    def amax(v):
        t = torch.tensor([v], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t[0])

    ms_local = 100.0 * (rank + 1)  # rank 1 is the slow one
    value, ms = bench.combine_ranks(ms_local, 1000, world, amax)
    out.put((rank, value, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms in res:
        assert ms == 200.0
        assert abs(value - 2 * 1000 / 0.2) < 1e-9
