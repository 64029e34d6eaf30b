"""Multi-process path: runs sharded over ranks with no data-path collective.

The sharding logic is host code, so it is checked on CPU with two ``gloo``
ranks: each rank simulates its cost-balanced share of an uneven batch of
density-matrix circuits (with the oracle standing in for the per-rank GPU
sweep, which is the same function of the same inputs), the shares are gathered
off the data path, and the reassembled batch must equal the single-process
result bit for bit.  The max-over-ranks timing reduction is checked too.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import socket
import tempfile

import numpy as np
import pytest
import torch

from mentpy_gb300 import circuit as C
from mentpy_gb300.plan import compile_plan
from mentpy_gb300.replicas import (dm_run_cost, gather_rows, partition_by_cost, rank_slice, reduce_max,
                                   scatter_back, shard_plans, sv_run_cost)

SHAPES = [(1, 3), (2, 4), (3, 3), (1, 5), (2, 3), (3, 4), (1, 4), (2, 5), (1, 6)]


def _circuits():
    return [C.many_wires([d] * w) if w > 1 else C.linear_cluster(d) for w, d in SHAPES]


def _inputs(circs, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for c in circs:
        a = rng.uniform(0, 2 * np.pi, len(c.trainable_nodes))
        n = len(c.input_nodes)
        v = rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)
        out.append((a, v / np.linalg.norm(v)))
    return out


def _rows(circs, idx, inputs):
    from oracle.sweep import run_dm

    cap = max(4 ** len(c.output_nodes) for c in circs)
    rows = np.zeros((len(idx), cap), dtype=np.complex128)
    for r, i in enumerate(idx):
        a, v = inputs[i]
        rho, _, _ = run_dm(circs[i], a, v, noise_p=0.01)
        rows[r, : rho.size] = rho.ravel()
    return rows


def test_rank_slice_covers_and_balances():
    for n in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            parts = [rank_slice(n, r, world) for r in range(world)]
            covered = np.concatenate([np.arange(n)[s] for s in parts])
            assert np.array_equal(covered, np.arange(n))
            sizes = [s.stop - s.start for s in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        rank_slice(10, 2, 2)


def test_partition_by_cost_is_exact_cover_and_near_optimal():
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 4, 8):
        costs = rng.integers(1, 1000, size=257).astype(float)
        parts = partition_by_cost(costs, world)
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(257))
        loads = [costs[p].sum() for p in parts]
        lower = max(costs.sum() / world, costs.max())
        assert max(loads) <= 4.0 / 3.0 * lower + costs.max() * 1e-12 + 1e-9
    assert [len(p) for p in partition_by_cost([], 3)] == [0, 0, 0]
    with pytest.raises(ValueError):
        partition_by_cost([1.0, -1.0], 2)


def test_plan_costs_and_shards():
    circs = _circuits()
    plans = [compile_plan(c, "dm") for c in circs]
    for c, p in zip(circs, plans):
        sv = compile_plan(c, "sv")
        assert dm_run_cost(p) > sv_run_cost(sv) > 0
    shards = [shard_plans(plans, r, 2) for r in range(2)]
    assert np.array_equal(np.sort(np.concatenate(shards)), np.arange(len(plans)))
    loads = [sum(dm_run_cost(plans[i]) for i in s) for s in shards]
    assert max(loads) <= 4.0 / 3.0 * max(sum(loads) / 2, max(dm_run_cost(p) for p in plans))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        circs = _circuits()
        plans = [compile_plan(c, "dm") for c in circs]
        inputs = _inputs(circs)
        shards = [shard_plans(plans, r, world) for r in range(world)]
        mine = _rows(circs, shards[rank], inputs)
        gathered = gather_rows(torch.as_tensor(mine))
        full = scatter_back(shards, gathered)
        t = reduce_max(1.5 + rank)
        if rank == 0:
            np.savez(out_path, full=full.numpy(), t=t, n_mine=len(shards[rank]))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_reassemble_single_process_result():
    circs = _circuits()
    inputs = _inputs(circs)
    expect = _rows(circs, range(len(circs)), inputs)
    ctx = mp.get_context("spawn")
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "r0.npz")
        port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        codes = [p.exitcode for p in procs]
        for p in procs:
            if p.is_alive():
                p.kill()
        assert codes == [0, 0], codes
        z = np.load(out)
        assert np.array_equal(z["full"], expect)
        assert float(z["t"]) == 2.5
        assert 0 < int(z["n_mine"]) < len(circs)


def test_single_process_helpers_without_group():
    x = torch.arange(6, dtype=torch.float32).reshape(3, 2)
    assert gather_rows(x) is x
    assert reduce_max(3.25) == 3.25
    shards = partition_by_cost([5.0, 1.0, 3.0], 2)
    g = torch.cat([torch.as_tensor(s, dtype=torch.float32)[:, None] for s in shards])
    back = scatter_back(shards, g)
    assert torch.equal(back[:, 0], torch.tensor([0.0, 1.0, 2.0]))


class _OracleFidelity:
    """Per-rank stand-in for ``StatevectorSweep.fidelity_grad`` on CPU."""

    def __init__(self, circuit):
        self.circuit = circuit
        self.n_angles = len(circuit.trainable_nodes)

    def fidelity_grad(self, angles, inputs, targets):
        from oracle.gradients import fidelity_grad, fidelity_loss

        A = np.atleast_2d(np.asarray(angles, dtype=float))
        loss = np.array([fidelity_loss(self.circuit, a, inputs, targets) for a in A])
        grad = np.stack([fidelity_grad(self.circuit, a, inputs, targets) for a in A])
        return torch.as_tensor(loss), torch.as_tensor(grad)


def _fid_problem():
    circ = C.linear_cluster(5)
    rng = np.random.default_rng(11)
    ang = rng.uniform(0, 2 * np.pi, size=(2, len(circ.trainable_nodes)))
    J = 5
    inp = rng.standard_normal((J, 2)) + 1j * rng.standard_normal((J, 2))
    inp /= np.linalg.norm(inp, axis=1, keepdims=True)
    tg = rng.standard_normal((J, 2)) + 1j * rng.standard_normal((J, 2))
    tg /= np.linalg.norm(tg, axis=1, keepdims=True)
    return circ, ang, inp, tg


def _fid_rank_main(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    from mentpy_gb300.replicas import sharded_fidelity_grad

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        circ, ang, inp, tg = _fid_problem()
        loss, grad = sharded_fidelity_grad(_OracleFidelity(circ), ang, inp, tg)
        np.savez(out_path + f".{rank}.npz", loss=loss.numpy(), grad=grad.numpy())
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_sharded_fidelity_gradient():
    circ, ang, inp, tg = _fid_problem()
    full_loss, full_grad = _OracleFidelity(circ).fidelity_grad(ang, inp, tg)
    ctx = mp.get_context("spawn")
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "fid")
        port = _free_port()
        procs = [ctx.Process(target=_fid_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=180)
        codes = [p.exitcode for p in procs]
        for p in procs:
            if p.is_alive():
                p.kill()
        assert codes == [0, 0], codes
        for r in range(2):
            z = np.load(out + f".{r}.npz")
            # same mean, split 3 + 2 over the ranks: agreement to rounding of the FD quotient
            np.testing.assert_allclose(z["loss"], full_loss.numpy(), rtol=0, atol=1e-12)
            np.testing.assert_allclose(z["grad"], full_grad.numpy(), rtol=0, atol=1e-9)
