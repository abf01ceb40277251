"""The multi-rank path on CPU: two gloo ranks shard a list of images, extract
their shards (with the CPU oracle standing in for the GPU worker) and gather
the rows; the result equals a single-process extraction, and the step time is
the slowest rank's."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

import synth_loader  # noqa: F401


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conftest import oracle_features, oracle_lib
    from gpu_helpers import images
    from wndcharm.dist import extract_sharded, max_over_ranks
    imgs = images(seed=13, sizes=[(24, 20), (17, 23), (30, 18), (16, 16), (21, 25)])
    lib = oracle_lib()
    rows = extract_sharded(imgs, lambda part: np.stack([oracle_features(lib, a) for a in part]))
    t = max_over_ranks(1.0 + rank)
    q.put((rank, rows, t))
    dist.destroy_process_group()


def test_shard_bounds():
    from wndcharm.dist import shard
    for n in range(0, 13):
        for world in range(1, 5):
            spans = [shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1


def test_two_gloo_ranks():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from conftest import oracle_features, oracle_lib
    from gpu_helpers import images
    imgs = images(seed=13, sizes=[(24, 20), (17, 23), (30, 18), (16, 16), (21, 25)])
    lib = oracle_lib()
    ref = np.stack([oracle_features(lib, a) for a in imgs])
    for rank, rows, t in res:
        np.testing.assert_array_equal(rows, ref)
        assert t == 2.0
