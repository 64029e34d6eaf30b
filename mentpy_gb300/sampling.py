"""Sampled outcomes with flow byproduct corrections (force0=False).

The reference's numpy simulators force every outcome to 0; its PennyLane
backend (pennylane_simulator.py:133-152) measures each node, and on outcome 1
applies X to flow(i) and Z to every neighbour of flow(i) measured after i.
``byproduct_tables`` turns a circuit's causal flow into the per-step tables
of ``mbqc_sv_forward_sampled`` (targets as lists, so any number of steps);
``StatevectorSweep.forward_sampled`` runs it.
"""
from __future__ import annotations

import numpy as np

from .plan import WindowPlan

__all__ = ["byproduct_tables"]


def byproduct_tables(circuit, plan: WindowPlan):
    """``(x_step int32 [M], z_off int32 [M + 1], z_idx int32 [nnz], x_out
    uint32 [M], z_out uint32 [M])``: the targets of each step's byproducts on
    outcome 1 -- steps by index (the Z targets of step k are
    ``z_idx[z_off[k]:z_off[k + 1]]``), outputs by their bit in the output
    index (output j = bit n_out-1-j)."""
    if circuit.flow is None:
        raise ValueError("sampled outcomes need a causal flow (MBQCircuit.flow is None)")
    M = plan.n_steps
    if plan.n_out > 32:
        raise ValueError(f"sampled outcomes support at most 32 output qubits, not {plan.n_out}")
    order = list(circuit.measurement_order)
    pos = {v: i for i, v in enumerate(order)}
    step_of = {v: k for k, v in enumerate(plan.schedule_measure)}
    out_bit = {v: plan.n_out - 1 - j for j, v in enumerate(plan.out_nodes)}
    x_step = np.full(M, -1, dtype=np.int32)
    z_off = np.zeros(M + 1, dtype=np.int32)
    z_idx = []
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
        targets = []
        for nb in g.neighbors(f):
            if nb == i or pos[nb] <= pos[i]:
                continue
            if nb in step_of:
                t = step_of[nb]
                if t <= k:
                    raise ValueError(f"neighbour {nb} of flow({i}) is measured before {i} in the window schedule")
                targets.append(t)
            elif nb in out_bit:
                z_out[k] |= np.uint32(1 << out_bit[nb])
        z_idx.extend(sorted(targets))
        z_off[k + 1] = len(z_idx)
    return x_step, z_off, np.asarray(z_idx, dtype=np.int32).reshape(-1), x_out, z_out
