"""Multi-rank host logic on CPU (gloo, world size 2): shot sharding with the
misfit/gradient sum, and the slowest-rank time the bench reports.  The data
path has no collective (replicas / independent shots), so a fake per-shot
gradient stands in for the GPU adjoint here."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


class _P:
    shape = (6, 5)
    family = 1  # seismic2


class _PEm:
    shape = (6, 5)
    family = 4  # electromag2


def _fake_gradient_em(p, shots, observed):
    loss = float(sum(s for s in shots))
    g = {k: sum((s + 1.0) * (q + 1) * np.ones(p.shape) for s in shots) for q, k in
         enumerate(("e11", "e13", "e33", "s11", "s13", "s33"))}
    return loss, g


def _worker_idle(rank, world, port, out):
    """One shot over `world` ranks: every rank but rank 0 owns no shot."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from seidart_gpu.distributed import sharded_gradient
        loss, g = sharded_gradient(_PEm(), [0], [None], rank, world, gradient=_fake_gradient_em)
        out.put((rank, loss, sorted(g), {k: float(v.sum()) for k, v in g.items()}))
    finally:
        dist.destroy_process_group()


def _fake_gradient(p, shots, observed):
    # per-shot contributions that depend on the shot index only
    loss = float(sum(s for s in shots))
    g = {k: sum((s + 1.0) * (q + 1) * np.ones(p.shape) for s in shots) for q, k in
         enumerate(("c11", "c13", "c33", "c55", "rho"))}
    return loss, g


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from seidart_gpu.distributed import reduce_max, shard, sharded_gradient
        shots = list(range(7))
        mine = shard(shots, rank, world)
        loss, g = sharded_gradient(_P(), shots, [None] * len(shots), rank, world, gradient=_fake_gradient)
        t = reduce_max(1.0 + rank)
        out.put((rank, mine, loss, {k: float(v.sum()) for k, v in g.items()}, t))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_gradient_and_max_time_world2():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    owned = sorted(s for r in res for s in r[1])
    assert owned == list(range(7))                       # every shot exactly once
    full_loss, full_g = _fake_gradient(_P(), list(range(7)), None)
    for rank, mine, loss, gsum, t in res:
        assert loss == full_loss                         # both ranks hold the full sum
        for k, v in full_g.items():
            assert gsum[k] == pytest.approx(v.sum())
        assert t == 2.0                                  # slowest rank


def test_sharded_gradient_idle_rank_electromag2():
    """More ranks than shots on an electromag2 inversion: the idle rank must
    contribute zeros under the EM gradient keys, so both ranks make the same
    collectives and return the one shot's loss and gradient."""
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_idle, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    full_loss, full_g = _fake_gradient_em(_PEm(), [0], None)
    for rank, loss, keys, gsum in res:
        assert keys == sorted(full_g)
        assert loss == full_loss
        for k, v in full_g.items():
            assert gsum[k] == pytest.approx(v.sum())


def test_shard_rejects_bad_rank():
    from seidart_gpu.distributed import shard
    with pytest.raises(ValueError):
        shard([1, 2], 2, 2)
