"""The reference algorithm, restated: dense 2^w x 2^w operators per step.

TEST AND CPU-BASELINE INFRASTRUCTURE ONLY (see ``oracle/__init__``).

mentpy's numpy statevector simulator expands every single-qubit projector and
every CZ to a dense matrix on the whole window with ``kron`` chains
(gates.py:62-72 ``arbitrary_qubit_gate``, gates.py:127-143 ``controlled_z``)
and applies them with matrix-vector products (np_simulator_sv.py:322-358,
207-223); the initial CZ layer is a product of such matrices built once in the
constructor (np_simulator_sv.py:112-128) and applied on every ``reset``
(np_simulator_sv.py:299-315).  This module performs the same operations, with
the same shapes, so that timing it on a host measures the reference algorithm
on that host.  ``DenseSV.run`` is one ``reset(input_state)`` + ``run(angles)``.
"""
from __future__ import annotations

import numpy as np

from .sweep import povm, schedule_for, _perm_state

_PLUS = np.array([1, 1], dtype=complex) / np.sqrt(2)


def embed(u, i, n):
    """u on qubit i of n (MSB first), identity elsewhere, as one dense matrix."""
    op = np.ones((1, 1))
    for k in range(n):
        op = np.kron(op, u if k == i else np.eye(2))
    return op


def dense_cz(i, j, n):
    """Dense CZ between qubits i and j of n: I - 2 |11><11|_{ij} (x) I."""
    one = np.array([[0, 0], [0, 1]])
    proj = np.ones((1, 1))
    for k in range(n):
        proj = np.kron(proj, one if k in (i, j) else np.eye(2))
    return np.eye(2**n) - 2 * proj


class DenseSV:
    """Dense-operator windowed statevector sweep (the reference's algorithm)."""

    def __init__(self, circuit, window_size=1, schedule=None):
        self.c = circuit
        self.sched, self.meas, self.w = schedule_for(circuit, "sv", window_size, schedule)
        self.N = circuit.graph.number_of_nodes()
        w = self.w
        win = self.sched[:w]
        init = np.eye(2**w)
        for a, na in enumerate(win):
            for nb in circuit.graph.neighbors(na):
                if nb in win and na < nb:
                    init = dense_cz(a, win.index(nb), w) @ init
        self.init = init
        self.trainable = list(circuit.trainable_nodes)

    def run(self, angles, input_state=None):
        c, w, N = self.c, self.w, self.N
        n_in = len(c.input_nodes)
        if input_state is None:
            input_state = np.ones(2**n_in, dtype=complex) / np.sqrt(2**n_in)
        psi = _perm_state(np.asarray(input_state, dtype=complex), list(c.input_nodes), self.sched[:n_in])
        for _ in range(w - n_in):
            psi = np.kron(psi, _PLUS)
        psi = self.init @ psi
        for k, node in enumerate(self.meas):
            ment = c[node]
            ang = angles[self.trainable.index(node)] if node in self.trainable else ment.angle
            n_cur = min(w, N - k)
            p0, p1 = povm(ment.plane, ang)
            p1e = embed(p1, 0, n_cur)
            p0e = embed(p0, 0, n_cur)
            _prob0 = np.dot(np.conj(psi), p0e @ psi)
            _prob1 = np.dot(np.conj(psi), p1e @ psi)
            psi = p0e @ psi
            psi = psi / np.linalg.norm(psi)
            psi = psi.reshape(2, -1).sum(axis=0)
            psi = psi / np.linalg.norm(psi)
            if k + 1 + w <= N:
                psi = np.kron(psi, _PLUS)
                win = self.sched[k + 1 : k + 1 + w]
                for nb in c.graph.neighbors(win[-1]):
                    if nb in win:
                        psi = dense_cz(win.index(nb), w - 1, w) @ psi
        M = len(self.meas)
        current = self.sched[M : M + w]
        if list(c.quantum_output_nodes) != current:
            psi = _perm_state(psi, current, list(c.output_nodes))
        return np.outer(psi, psi.conj())
