"""Candidate sharding across ranks (one process per GPU): world size 2 over gloo
on CPU, with the CPU oracle standing in for each rank's GPU evaluation.  The
gathered INFO rows equal a single-process evaluation, in candidate order."""
import os
import socket

import numpy as np
import pytest

from controllerengine_gb300.distributed import shard_bounds


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 7, 1536, 65536, 1001):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from controllerengine_gb300 import synth
        from controllerengine_gb300.distributed import evaluate_sharded
        from oracle import oracle as O
        p = synth.mass_spring(1536)
        orc = O.Oracle(p.config_text, p.plant, threads=2)
        n = 301  # not a multiple of the world size
        out = evaluate_sharded(lambda g, i: orc.evaluate(g, i), p.cuda_mx[:n], p.info_mx[:n])
        if rank == 0:
            q.put(out)
    finally:
        dist.destroy_process_group()


def test_gather_matches_single_process():
    import multiprocessing as mp
    from controllerengine_gb300 import synth
    from oracle import oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    p = synth.mass_spring(1536)
    ref = O.Oracle(p.config_text, p.plant, threads=2).evaluate(p.cuda_mx[:301], p.info_mx[:301])
    assert np.array_equal(out, ref, equal_nan=True)
