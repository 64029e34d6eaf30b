"""complex128 gradient references for the adjoint kernels -- TEST INFRASTRUCTURE ONLY.

The reference has no autodiff; its gradients are central finite differences of
the whole simulation (mentpy/gradients/_finite_difference.py:9-25).  This
module evaluates the same costs on the complex128 restatement
(``oracle.sweep``) and differentiates them by central differences.
"""
from __future__ import annotations

import numpy as np

from . import sweep


def ref_phase(circuit, angles, window_size=1, schedule=None):
    """Global phase the reference's summing partial trace puts on the
    statevector output: prod over measured steps of (v0 + v1)/|v0 + v1|
    (state_ops.py:69,73), v = the outcome-0 eigenvector of the step."""
    _, meas, _ = sweep.schedule_for(circuit, "sv", window_size, schedule)
    trainable = list(circuit.trainable_nodes)
    ph = 1.0 + 0j
    for node in meas:
        m = circuit[node]
        theta = angles[trainable.index(node)] if node in trainable else m.angle
        p0, _ = sweep.povm(m.plane, theta)
        v0 = np.sqrt(p0[0, 0].real)
        v = np.array([v0, p0[1, 0] / v0])
        s = v[0] + v[1]
        ph *= s / abs(s)
    return ph


def canonical_sv(circuit, angles, psi_in=None, **kw):
    """Normalised output state without the reference global phase."""
    st, _, _ = sweep.run_sv(circuit, angles, psi_in, output_form="sv", **kw)
    return st * np.conj(ref_phase(circuit, angles, **kw))


def central_fd(f, x, h=1e-5):
    x = np.asarray(x, dtype=float)
    g = np.zeros(len(x))
    for i in range(len(x)):
        e = np.zeros(len(x))
        e[i] = h
        g[i] = (f(x + e) - f(x - e)) / (2 * h)
    return g


def linear_functional_grad(circuit, angles, psi_in, gout, h=1e-5, **kw):
    """d/dangles of Re sum conj(gout) z(angles): the quantity the generic adjoint returns."""
    f = lambda a: float(np.real(np.vdot(gout, canonical_sv(circuit, a, psi_in, **kw))))  # noqa: E731
    return central_fd(f, angles, h)


def dm_linear_functional_grad(circuit, angles, psi_in, gamma, noise_p=0.0, h=1e-5, **kw):
    """d/dangles of Re sum conj(gamma) rho_out(angles) for the (noisy)
    density-matrix sweep: what the density-matrix adjoint returns."""
    def f(a):
        rho, _, _ = sweep.run_dm(circuit, a, psi_in, noise_p=noise_p, **kw)
        return float(np.real(np.vdot(gamma, rho)))

    return central_fd(f, angles, h)


def fidelity_loss(circuit, angles, inputs, targets, **kw):
    """1 - mean_j |<t_j | z(angles, psi_j)>|^2 (docs/tutorials/intro-to-mbqml.rst:35-54)."""
    F = [abs(np.vdot(t, canonical_sv(circuit, angles, p, **kw))) ** 2 for p, t in zip(inputs, targets)]
    return 1.0 - float(np.mean(F))


def fidelity_grad(circuit, angles, inputs, targets, h=1e-5, **kw):
    return central_fd(lambda a: fidelity_loss(circuit, a, inputs, targets, **kw), angles, h)


def fidelity_losses(circuit, angle_rows, inputs, targets, chunk_runs=65536, **kw):
    """``fidelity_loss`` for every row of ``angle_rows`` [V, A], vectorised
    over all V x J runs (``sweep.run_sv_batch``; the fidelity ignores the
    global phase)."""
    angle_rows = np.atleast_2d(np.asarray(angle_rows, dtype=float))
    inputs = np.asarray(inputs, dtype=complex)
    targets = np.asarray(targets, dtype=complex)
    V, J = angle_rows.shape[0], inputs.shape[0]
    per = max(1, chunk_runs // J)
    out = np.empty(V)
    for v0 in range(0, V, per):
        rows = angle_rows[v0 : v0 + per]
        n = rows.shape[0]
        st, _ = sweep.run_sv_batch(circuit, np.repeat(rows, J, axis=0), np.tile(inputs, (n, 1)), **kw)
        ov = np.einsum("rj,rj->r", np.tile(targets, (n, 1)).conj(), st).reshape(n, J)
        out[v0 : v0 + n] = 1.0 - np.mean(np.abs(ov) ** 2, axis=1)
    return out


def fidelity_grad_fd(circuit, angles, inputs, targets, h=1e-4, **kw):
    """Central finite-difference gradient of ``fidelity_loss`` at one angle
    vector (mentpy's fd_gradient, gradients/_finite_difference.py:9-25), all
    2A shifted evaluations in one vectorised batch."""
    x = np.asarray(angles, dtype=float)
    A = len(x)
    rows = np.repeat(x[None], 2 * A, axis=0)
    rows[np.arange(A), np.arange(A)] += h
    rows[A + np.arange(A), np.arange(A)] -= h
    f = fidelity_losses(circuit, rows, inputs, targets, **kw)
    return (f[:A] - f[A:]) / (2 * h)
