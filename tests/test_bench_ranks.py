"""The multi-replica figures of bench.py, on CPU: two gloo ranks with different
step times combine into the slowest rank's time and units x world over it,
for the device-timed figure and for the end-to-end one (the replicas share no
data; the one collective is this reduction)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    res = {"ms_per_step": 10.0 + 5.0 * rank, "value": 0.0, "e2e": {"ms_per_step": 20.0 + rank, "value": 0.0}}
    out = bench.combine_over_ranks(res, 1000, world, device="cpu")
    q.put((rank, out))
    torch.distributed.destroy_process_group()


def test_combine_over_ranks_gloo():
    import torch.multiprocessing as mp

    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    outs = dict(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        assert outs[r]["ms_per_step"] == 15.0
        assert outs[r]["value"] == pytest.approx(1000 * world / 15e-3)
        assert outs[r]["e2e"]["ms_per_step"] == 21.0
        assert outs[r]["e2e"]["value"] == pytest.approx(1000 * world / 21e-3)


def test_single_rank_is_unchanged():
    import bench

    res = {"ms_per_step": 3.0, "value": 7.0}
    assert bench.combine_over_ranks(res, 10, 1) is res and res["value"] == 7.0
