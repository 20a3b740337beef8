"""The multi-GPU form is replicas only: each rank traces its own inputs on its
own GPU and bench.py aggregates the whole job -- units summed, time maximised
over ranks.  That host logic runs here with two gloo ranks on CPU."""
import os
import socket

import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        w, r, local = bench.dist_setup()
        units, sec = bench.across_ranks(1000 * (rank + 1), 0.5 + rank, dist, torch.device("cpu"))
        dist.barrier()
        q.put((r, w, local, units, sec))
    finally:
        dist.destroy_process_group()


def test_replicas_aggregate_over_two_gloo_ranks():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(ws))
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, local, units, sec in out:
        assert w == 2 and local == r
        assert units == 3000.0 and sec == 1.5


def test_single_process_passes_values_through():
    import bench

    assert bench.across_ranks(123, 0.25, None, None) == (123, 0.25)
