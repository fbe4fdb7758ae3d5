"""The multi-process path on CPU ranks (torch.distributed, gloo, world size 2): shard ranges, view
partitions, the framebuffer gather, and the data-parallel gradient average of the learned proposal
checked against the CPU network oracle on the union of the ranks' batches."""
import os
import socket

import numpy as np
import pytest

from pltfalcor_gb300 import distributed as D

WORLD = 2


def test_shard_range_covers_everything_once():
    for n in (0, 1, 7, 1 << 22, 1000003):
        for world in (1, 2, 3, 8):
            spans = [D.shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1


def test_partition_views_balances_paths():
    rng = np.random.default_rng(3)
    px = (np.exp(rng.uniform(np.log(4096), np.log(1 << 20), 64))).astype(np.int64)
    for world in (2, 4, 8):
        parts = D.partition_views(px, world)
        assert sorted(v for p in parts for v in p) == list(range(64))
        loads = [int(px[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= px.max()      # greedy bound: one view at most


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, queue):
    import sys
    import torch
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import oracle
    try:
        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=WORLD)
        # framebuffers: each rank renders its share of 5 views (synthetic images), rank 0 gathers
        px = [64 * 64, 32 * 32, 128 * 96, 16 * 16, 48 * 48]
        mine = D.partition_views(px, WORLD)[rank]
        local = {v: np.full((4, 4, 4), float(v) + 0.25, np.float32) for v in mine}
        allimg = D.gather_images(local, dist)
        # data-parallel gradient: each rank's batch, averaged, vs the oracle on both batches
        rng = np.random.default_rng(11)
        params = (rng.standard_normal(11488) * 0.1).astype(np.float32)
        n = 64
        xs = [rng.standard_normal((n, 16)).astype(np.float32) for _ in range(WORLD)]
        ts = [rng.uniform(0, 1, (n, 2)).astype(np.float32) for _ in range(WORLD)]
        ws = [rng.uniform(0, 2, n).astype(np.float32) for _ in range(WORLD)]
        bits = lambda x: (x.view(np.uint32) >> 16).astype(np.uint16)   # truncation to bf16 bits
        loss, g = oracle.mlp_gradient(params, ts[rank], ws[rank], x_bits=bits(xs[rank]))
        gt = torch.from_numpy(np.asarray(g, np.float64).copy())
        D.allreduce_mean_(gt, dist)
        if rank == 0:
            _, gall = oracle.mlp_gradient(params, np.concatenate(ts), np.concatenate(ws), x_bits=bits(np.concatenate(xs)))
            queue.put(("ok", sorted(allimg.keys()), {k: float(v.mean()) for k, v in allimg.items()},
                       float(np.abs(gt.numpy() - gall).max()), float(np.abs(gall).max())))
        dist.barrier()
        dist.destroy_process_group()
    except Exception as e:   # reported to the parent, which fails the test
        queue.put(("error", repr(e)))


def test_two_rank_gather_and_gradient_average(oracle_lib):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(WORLD)]
    for p in procs:
        p.start()
    try:
        res = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert res[0] == "ok", res
    _, keys, means, gerr, gmax = res
    assert keys == [0, 1, 2, 3, 4]
    assert all(abs(means[k] - (k + 0.25)) < 1e-6 for k in keys)
    assert gerr <= 1e-9 * max(1.0, gmax), (gerr, gmax)
