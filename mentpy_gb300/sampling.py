"""Sampled outcomes with flow byproduct corrections (force0=False).

The reference's numpy simulators force every outcome to 0; its PennyLane
backend (pennylane_simulator.py:133-152) measures each node, and on outcome 1
applies X to flow(i) and Z to every neighbour of flow(i) measured after i.
``byproduct_tables`` turns a circuit's causal flow into the per-step tables
of ``mbqc_sv_forward_sampled``; ``StatevectorSweep.forward_sampled`` runs it.
"""
from __future__ import annotations

import numpy as np

from .plan import WindowPlan

__all__ = ["byproduct_tables"]


def byproduct_tables(circuit, plan: WindowPlan):
    """``(x_step int16 [M], z_steps uint64 [M, 2], x_out uint32 [M], z_out
    uint32 [M])``: the targets of each step's byproducts on outcome 1 (steps
    by index, outputs by their bit in the output index, output j = bit
    n_out-1-j)."""
    if circuit.flow is None:
        raise ValueError("sampled outcomes need a causal flow (MBQCircuit.flow is None)")
    M = plan.n_steps
    if M > 128:
        raise ValueError(f"sampled outcomes support at most 128 measured nodes, not {M}")
    order = list(circuit.measurement_order)
    pos = {v: i for i, v in enumerate(order)}
    step_of = {v: k for k, v in enumerate(plan.schedule_measure)}
    out_bit = {v: plan.n_out - 1 - j for j, v in enumerate(plan.out_nodes)}
    x_step = np.full(M, -1, dtype=np.int16)
    z_steps = np.zeros((M, 2), dtype=np.uint64)
    x_out = np.zeros(M, dtype=np.uint32)
    z_out = np.zeros(M, dtype=np.uint32)
    g = circuit.graph
    for k, i in enumerate(plan.schedule_measure):
        f = circuit.flow(i)
        if f in step_of:
            if step_of[f] <= k:
                raise ValueError(f"flow({i}) = {f} is measured before {i}")
            x_step[k] = step_of[f]
        elif f in out_bit:
            x_out[k] |= np.uint32(1 << out_bit[f])
        else:
            raise ValueError(f"flow({i}) = {f} is neither measured nor an output")
        for nb in g.neighbors(f):
            if nb == i or pos[nb] <= pos[i]:
                continue
            if nb in step_of:
                t = step_of[nb]
                z_steps[k, t >> 6] |= np.uint64(1 << (t & 63))
            elif nb in out_bit:
                z_out[k] |= np.uint32(1 << out_bit[nb])
    return x_step, z_steps, x_out, z_out
