"""Replica sharding over 2 CPU ranks (gloo): row bands rendered by the CPU
restatement and gathered equal the single-rank image, and averaging
per-rank cache gradients equals the gradient of the whole batch."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from kiraray_gb300 import sharding


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, task, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = task(rank, world)
    finally:
        dist.barrier()
        dist.destroy_process_group()


def _run(task, world=2):
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, task, out), nprocs=world, join=True)
        return dict(out)


def _render_band(rank, world):
    from kiraray_gb300 import scenes
    from oracle import pyoracle as O
    sc = scenes.cornell_box(32, 24, max_depth=3)
    b, e = sharding.row_band(sc.width, sc.height, rank, world)
    L, _ = O.PathTracer(sc).render({"max_depth": 3}, 1, b, e)
    full = sharding.gather_rows(torch.from_numpy(L), sc.width, sc.height, rank, world)
    return None if full is None else full.numpy()


def test_row_bands_cover_the_image():
    for w, h, n in ((7, 5, 2), (32, 24, 3), (1, 1, 1), (4, 9, 4)):
        bands = [sharding.row_band(w, h, r, n) for r in range(n)]
        assert bands[0][0] == 0 and bands[-1][1] == w * h
        assert all(bands[i][1] == bands[i + 1][0] for i in range(n - 1))
        sizes = [e - b for b, e in bands]
        assert max(sizes) - min(sizes) <= w
    with pytest.raises(ValueError):
        sharding.row_band(4, 4, 2, 2)


def test_two_rank_gather_equals_single_rank(oracle_lib):
    out = _run(_render_band)
    from kiraray_gb300 import scenes
    from oracle import pyoracle as O
    sc = scenes.cornell_box(32, 24, max_depth=3)
    want, _ = O.PathTracer(sc).render({"max_depth": 3}, 1)
    assert out[1] is None
    assert np.array_equal(out[0], want)


def _grad_shards(rank, world):
    import types
    from oracle import nrc_ref as R
    rng = np.random.default_rng(0)
    info = types.SimpleNamespace(n_levels=2, resolution=[2, 4], level_offset=[0, 27],
                                 level_size=[27, 64])
    grid = R.Grid(info, [0, 0, 0], [1, 1, 1], table_size=64)
    table = rng.normal(size=91 * 2) * 0.2
    mlp = R.Mlp(rng.normal(size=2 * R.WIDTH * R.IN + R.OUT_PAD * R.IN) * 0.2, 3)
    inp = rng.random((64, 13))
    t = rng.random((64, 3))
    shard = slice(rank * 32, rank * 32 + 32)

    def grads(x, tt):
        X0, cs = R.encode(grid, table, x, rounding=False)
        y, acts = R.forward(mlp, X0, rounding=False)
        _, dy = R.loss_and_grad(y, tt)
        gW, _ = R.backward(mlp, acts, dy, rounding=False)
        return np.concatenate([g.reshape(-1) for g in gW])

    local = torch.from_numpy(grads(inp[shard], t[shard]))
    avg = sharding.allreduce_mean(local, world).numpy()
    return avg, grads(inp, t)


def test_gradient_allreduce_equals_full_batch():
    out = _run(_grad_shards)
    for rank in (0, 1):
        avg, full = out[rank]
        assert np.allclose(avg, full, rtol=1e-10, atol=1e-14)
