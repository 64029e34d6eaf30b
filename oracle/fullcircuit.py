"""Whole-graph density-matrix simulation with depolarising noise -- TEST INFRASTRUCTURE ONLY.

Restates the circuit mentpy's PennyLane backend builds
(mentpy/simulators/pennylane_simulator.py:97-166) for small graphs, in numpy:
the input state on the input nodes, |+> on the others (Hadamard on |0>), a CZ
on every edge, one depolarising channel on every qubit after the CZ layer
(:123-126), then every non-output node measured in measurement order by
RZ(-theta), H and a Z measurement (:138-143).  With every outcome post-selected
to 0 the byproduct corrections (:144-153) are never applied, which is what the
numpy simulators' force0 sweep computes.  The windowed sweep with noise applied
to each qubit right before it is measured (and to the outputs at the end) must
agree with this whenever the window holds every CZ partner of a node before
the node is measured; ``tests/test_dm_noise.py`` checks that.

PennyLane itself is not installed here, so this restatement, not PennyLane,
is the check (noisy parity is unpinned against the reference code).
"""
from __future__ import annotations

import numpy as np

from .sweep import povm


def _apply(rho, op, q, n):
    d = 2**n
    t = rho.reshape([2] * (2 * n))
    t = np.moveaxis(np.tensordot(op, t, axes=([1], [q])), 0, q)
    t = np.moveaxis(np.tensordot(t, op.conj().T, axes=([n + q], [0])), -1, n + q)
    return t.reshape(d, d)


def _depolarise(rho, q, n, p):
    X = np.array([[0, 1], [1, 0]], complex)
    Y = np.array([[0, -1j], [1j, 0]], complex)
    Z = np.array([[1, 0], [0, -1]], complex)
    out = (1 - p) * rho
    for P in (X, Y, Z):
        out = out + (p / 3) * _apply(rho, P, q, n)
    return out


def run_full_dm(circuit, angles, input_state=None, noise_p=0.0):
    """rho over ``output_nodes`` (in that order) of the post-selected circuit."""
    nodes = sorted(circuit.graph.nodes())
    n = len(nodes)
    pos = {v: i for i, v in enumerate(nodes)}
    n_in = len(circuit.input_nodes)
    if input_state is None:
        input_state = np.ones(2**n_in) / np.sqrt(2**n_in)
    plus = np.array([1, 1], complex) / np.sqrt(2)
    # |psi> = input on input nodes (in input order), |+> elsewhere, kron in node order
    t = np.asarray(input_state, complex).reshape([2] * n_in)
    rest = [v for v in nodes if v not in circuit.input_nodes]
    for _ in rest:
        t = np.multiply.outer(t, plus)
    order = list(circuit.input_nodes) + rest
    t = np.transpose(t, [order.index(v) for v in nodes])
    psi = t.reshape(-1)
    idx = np.arange(2**n)
    for a, b in circuit.graph.edges():
        ba = (idx >> (n - 1 - pos[a])) & 1
        bb = (idx >> (n - 1 - pos[b])) & 1
        psi = psi * np.where(ba & bb, -1.0, 1.0)
    rho = np.outer(psi, psi.conj())
    for v in nodes:
        if noise_p:
            rho = _depolarise(rho, pos[v], n, noise_p)
    trainable = list(circuit.trainable_nodes)
    alive = list(nodes)
    for node in circuit.measurement_order:
        if node in circuit.output_nodes:
            continue
        m = circuit[node]
        theta = angles[trainable.index(node)] if node in trainable else m.angle
        p0, _ = povm(m.plane, theta)
        q = alive.index(node)
        k = len(alive)
        rho = _apply(rho, p0, q, k)
        rho = rho / np.trace(rho).real
        t = rho.reshape([2] * (2 * k))
        t = np.trace(t, axis1=q, axis2=k + q)
        alive.remove(node)
        rho = t.reshape(2 ** len(alive), 2 ** len(alive))
    perm = [alive.index(v) for v in circuit.output_nodes]
    k = len(alive)
    t = rho.reshape([2] * (2 * k))
    t = np.transpose(t, perm + [k + i for i in perm])
    return t.reshape(2**k, 2**k)


def run_full_sampled_sv(circuit, angles, input_state, outcomes, output_order):
    """Pure output state of the PennyLane backend's circuit
    (pennylane_simulator.py:114-153) with the mid-circuit outcomes given:
    input on the input nodes, |+> elsewhere, CZ on every edge, then each
    non-output node in measurement order: RZ(-theta), H, the outcome
    ``outcomes[node]`` projected, and on outcome 1 an X on flow(node) and a Z
    on every neighbour of flow(node) measured after node.  Returns the
    normalised amplitudes over ``output_order`` (first output = most
    significant bit)."""
    nodes = sorted(circuit.graph.nodes())
    n = len(nodes)
    pos = {v: i for i, v in enumerate(nodes)}
    n_in = len(circuit.input_nodes)
    if input_state is None:
        input_state = np.ones(2**n_in) / np.sqrt(2**n_in)
    plus = np.array([1, 1], complex) / np.sqrt(2)
    t = np.asarray(input_state, complex).reshape([2] * n_in)
    rest = [v for v in nodes if v not in circuit.input_nodes]
    for _ in rest:
        t = np.multiply.outer(t, plus)
    order = list(circuit.input_nodes) + rest
    t = np.transpose(t, [order.index(v) for v in nodes])
    idx = np.arange(2**n)
    bit = lambda v: (idx >> (n - 1 - pos[v])) & 1  # noqa: E731
    psi = t.reshape(-1).copy()
    for a, b in circuit.graph.edges():
        psi = psi * np.where(bit(a) & bit(b), -1.0, 1.0)
    H = np.array([[1, 1], [1, -1]], complex) / np.sqrt(2)
    X = np.array([[0, 1], [1, 0]], complex)
    Z = np.array([[1, 0], [0, -1]], complex)

    def op1(state, U, v):
        s = state.reshape([2] * n)
        s = np.moveaxis(np.tensordot(U, s, axes=([1], [pos[v]])), 0, pos[v])
        return s.reshape(-1)

    trainable = list(circuit.trainable_nodes)
    mo = list(circuit.measurement_order)
    for node in mo:
        if node in circuit.output_nodes:
            continue
        m = circuit[node]
        if m.plane == "XY":
            theta = angles[trainable.index(node)] if node in trainable else m.angle
        elif m.plane == "X":
            theta = 0.0
        elif m.plane == "Y":
            theta = np.pi / 2
        else:
            raise ValueError("XY, X and Y measurements only")
        rz = np.diag([np.exp(1j * theta / 2), np.exp(-1j * theta / 2)])  # RZ(-theta)
        psi = op1(op1(psi, rz, node), H, node)
        o = int(outcomes[node])
        psi = np.where(bit(node) == o, psi, 0)
        psi = psi / np.linalg.norm(psi)
        if o:
            f = circuit.flow(node)
            psi = op1(psi, X, f)
            for nb in circuit.graph.neighbors(f):
                if nb != node and mo.index(nb) > mo.index(node):
                    psi = op1(psi, Z, nb)
    # measured qubits sit in their outcome states: read the outputs' amplitudes
    sel = np.ones(2**n, bool)
    for node in mo:
        if node not in circuit.output_nodes:
            sel &= bit(node) == int(outcomes[node])
    out = np.zeros(2 ** len(output_order), complex)
    k = len(output_order)
    y = np.zeros(2**n, int)
    for j, v in enumerate(output_order):
        y |= bit(v) << (k - 1 - j)
    out[y[sel]] = psi[sel]
    return out / np.linalg.norm(out)
