"""Several processes, one GPU each: independent replicas and shot sharding.

The solvers have no exchange step (each model, and each shot of an
inversion, advances independently), so more GPUs means more independent
work: every rank runs its own replica or its own share of the shots, with
no collective on the data path.  The only collectives are on the host side
of a measurement or an inversion step: the slowest rank's time (MAX) and
the sum of per-shot misfits and gradients (SUM), through torch.distributed
(NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def shard(items: list, rank: int, world: int) -> list:
    """Round-robin share of ``items`` owned by ``rank`` (every item exactly once)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return items[rank::world]


def sharded_batch(problems: list, rank: int, world: int, **batch_kw):
    """This rank's share of a ragged batch (models round-robin over ranks) as
    one ``Batch`` on this rank's GPU, or None when the rank owns no model.
    Model m of ``problems`` is model ``m // world`` of rank ``m % world``'s
    batch; no collective is needed while the batches step."""
    from .batch import Batch
    mine = shard(problems, rank, world)
    return Batch(mine, **batch_kw) if mine else None


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def _device():
    import torch
    dist = _dist()
    if dist is not None and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def reduce_max(x: float) -> float:
    """Maximum of ``x`` over ranks (the slowest rank's time); ``x`` alone
    without an initialised process group."""
    import torch
    dist = _dist()
    if dist is None:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(arrays: dict) -> dict:
    """Elementwise sum over ranks of a dict of FP64 arrays (same keys and
    shapes on every rank)."""
    import torch
    dist = _dist()
    if dist is None:
        return {k: np.array(v, dtype=np.float64) for k, v in arrays.items()}
    out = {}
    for k in sorted(arrays):
        t = torch.as_tensor(np.ascontiguousarray(arrays[k], dtype=np.float64)).to(_device())
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        out[k] = t.cpu().numpy()
    return out


def sharded_gradient(problem, shots: list, observed: list, rank: int, world: int,
                     gradient: Callable | None = None, full_tensor: bool = False) -> tuple[float, dict]:
    """Misfit and gradient over all shots with each rank computing its share.

    ``gradient(problem, shots, observed) -> (loss, {name: array})`` defaults
    to the GPU adjoint (:class:`seidart_gpu.fwi.Fwi`).  The per-rank losses and
    gradients are summed over ranks, so every rank returns the full-batch
    result.  ``full_tensor`` (seismic2) adds dL/dc15 and dL/dc35."""
    if gradient is None:
        from .fwi import Fwi

        def gradient(p, s, o):
            with Fwi(p, s, o, full_tensor=full_tensor) as f:
                return f.gradient()

    idx = shard(list(range(len(shots))), rank, world)
    if idx:
        loss, g = gradient(problem, [shots[i] for i in idx], [observed[i] for i in idx])
    else:
        # a rank without shots still joins every collective: it sends zeros
        # under the same keys the busy ranks send for this problem family
        from .fwi import grad_keys
        loss, g = 0.0, {k: np.zeros(problem.shape, order="F") for k in grad_keys(problem.family, full_tensor)}
    arrays = {k: np.asarray(v, dtype=np.float64) for k, v in g.items()}
    arrays["__loss__"] = np.array([loss], dtype=np.float64)
    tot = allreduce_sum(arrays)
    loss = float(tot.pop("__loss__")[0])
    shape = problem.shape
    return loss, {k: v.reshape(shape, order="F") if v.ndim == 1 else v for k, v in tot.items()}
