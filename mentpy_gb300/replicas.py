"""Partition of independent MBQC runs over ranks (one process per GPU).

Every run of the windowed sweep (an angle vector, an input state, a circuit)
is independent of every other run, so a multi-GPU job shards the runs -- or
the circuits of an uneven batch -- across ranks and runs each shard on its own
GPU with no collective on the data path (weak scaling).  Collectives appear
only around the data path: the max-over-ranks step time of a benchmark, and
an optional gather of results for callers that want them on one rank.

The reference has no multi-process path (``pattern_simulator.py`` runs one
simulator per process); this module is the layer a data-parallel caller puts
above ``StatevectorSweep`` / ``UnevenDensityMatrixBatch``.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np
import torch

from .plan import WindowPlan


def rank_slice(n_units: int, rank: int, world: int) -> slice:
    """Contiguous, balanced share of ``n_units`` equal-cost runs for ``rank``:
    the first ``n_units % world`` ranks take one extra run."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    if n_units < 0:
        raise ValueError("negative number of runs")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def sv_run_cost(plan: WindowPlan) -> float:
    """Amplitude updates of one statevector run: sum over steps of the live
    window's 2^n amplitudes."""
    return float(sum(2 ** min(plan.window, plan.n_nodes - k) for k in range(plan.n_steps)) + 2 ** plan.n_out)


def dm_run_cost(plan: WindowPlan) -> float:
    """Entry updates of one density-matrix run: sum over steps of 4^n."""
    return float(sum(4 ** min(plan.window, plan.n_nodes - k) for k in range(plan.n_steps)) + 4 ** plan.n_out)


def partition_by_cost(costs: Sequence[float], world: int) -> List[np.ndarray]:
    """Split items of unequal cost over ``world`` ranks: longest processing
    time first (each item, largest first, goes to the least-loaded rank; ties
    to the lower rank), which keeps the largest rank load within 4/3 of the
    optimum.  Returns one sorted index array per rank; deterministic, so
    every rank computes the same partition without communicating."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    c = np.asarray(costs, dtype=np.float64)
    if c.ndim != 1:
        raise ValueError("costs must be one-dimensional")
    if (c < 0).any() or not np.isfinite(c).all():
        raise ValueError("costs must be finite and non-negative")
    order = np.argsort(-c, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(c), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))  # first minimum: lowest rank on ties
        owner[i] = r
        load[r] += c[i]
    return [np.flatnonzero(owner == r) for r in range(world)]


def shard_plans(plans: Sequence[WindowPlan], rank: int, world: int) -> np.ndarray:
    """Indices of the circuits of an uneven batch that ``rank`` simulates,
    balanced by each plan's simulation cost (density matrix or statevector,
    from ``plan.kind``)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    costs = [dm_run_cost(p) if p.kind == "dm" else sv_run_cost(p) for p in plans]
    return partition_by_cost(costs, world)[rank]


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def _coll_device(group=None) -> torch.device:
    dist = _dist()
    if dist is not None and dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def reduce_max(value: float, group=None) -> float:
    """Maximum of ``value`` over the ranks of ``group`` (the value itself
    without an initialised process group)."""
    dist = _dist()
    if dist is None:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=_coll_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_rows(local: torch.Tensor, group=None) -> torch.Tensor:
    """Concatenate every rank's rows (dim 0, any per-rank count, the same
    trailing shape and dtype) in rank order, on every rank.  Off the data
    path: for callers that want a sharded batch's results in one place."""
    dist = _dist()
    if dist is None:
        return local
    dev = _coll_device(group)
    world = dist.get_world_size(group)
    x = local.to(dev)
    n = torch.tensor([x.shape[0]], dtype=torch.int64, device=dev)
    counts = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    counts = [int(c.item()) for c in counts]
    cap = max(counts) if counts else 0
    if x.is_complex():
        x = torch.view_as_real(x)
    pad = torch.zeros((cap,) + tuple(x.shape[1:]), dtype=x.dtype, device=dev)
    pad[: x.shape[0]] = x
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    out = torch.cat([p[:c] for p, c in zip(parts, counts)], dim=0)
    if local.is_complex():
        out = torch.view_as_complex(out.contiguous())
    return out.to(local.device)


def scatter_back(shards: Sequence[np.ndarray], gathered: torch.Tensor) -> torch.Tensor:
    """Undo a cost partition: ``gathered`` holds rank 0's rows, then rank 1's,
    ... in the order of ``shards``; returns the rows in original item order."""
    order = np.concatenate([np.asarray(s, dtype=np.int64) for s in shards]) if shards else np.zeros(0, np.int64)
    if len(order) != gathered.shape[0]:
        raise ValueError("gathered rows do not match the partition")
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    return gathered[torch.as_tensor(inv, device=gathered.device)]


def allreduce_sum_(t: torch.Tensor, group=None) -> torch.Tensor:
    """In-place sum of ``t`` over the ranks of ``group`` (no-op without an
    initialised process group)."""
    dist = _dist()
    if dist is None:
        return t
    dev = _coll_device(group)
    x = t if t.device == dev else t.to(dev)
    dist.all_reduce(x, op=dist.ReduceOp.SUM, group=group)
    if x is not t:
        t.copy_(x)
    return t


def sharded_fidelity_grad(sweep, angles, inputs, targets, *, rank: Optional[int] = None,
                          world: Optional[int] = None, group=None):
    """Fidelity loss 1 - mean_j |<t_j|z(angles_v, psi_j)>|^2 and its gradient
    with the inputs (j) sharded over ranks.

    The loss is a mean over inputs, so every rank runs ``sweep.fidelity_grad``
    on its contiguous share of the inputs, weights its loss and gradient by
    its share of the inputs, and one all-reduce (sum) of the packed
    ``[V, 1 + A]`` block gives every rank the full result.  ``sweep`` is a
    ``StatevectorSweep`` (or any object with the same ``fidelity_grad`` and
    ``n_angles``).  Returns ``(loss [V], grad [V, A])`` float64.
    """
    dist = _dist()
    if rank is None:
        rank = dist.get_rank(group) if dist is not None else 0
    if world is None:
        world = dist.get_world_size(group) if dist is not None else 1
    ang = torch.as_tensor(angles)
    V = 1 if ang.dim() == 1 else ang.shape[0]
    J = len(inputs)
    if J == 0 or len(targets) != J:
        raise ValueError("inputs and targets must be non-empty and of equal length")
    s = rank_slice(J, rank, world)
    n_local = s.stop - s.start
    packed = torch.zeros((V, 1 + sweep.n_angles), dtype=torch.float64)
    if n_local > 0:
        loss, grad = sweep.fidelity_grad(angles, inputs[s], targets[s])
        packed[:, 0] = torch.as_tensor(loss).reshape(V).cpu()
        packed[:, 1:] = torch.as_tensor(grad).reshape(V, -1).cpu()
        packed *= n_local / J
    allreduce_sum_(packed, group)
    return packed[:, 0].clone(), packed[:, 1:].clone()
