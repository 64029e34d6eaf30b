"""Gradient and Hessian helpers with mentpy's signatures (mentpy/gradients/grad.py:13-60).

``fd_gradient`` and ``psr_gradient`` evaluate a black-box cost 2*len(x) times,
exactly like the reference (_finite_difference.py:9-25, _parameter_shift.py:9-25:
its "parameter shift" is a central difference with shift 1.5).  With a cost
built on ``PatternSimulator(..., backend="cuda-sv")`` each evaluation is one
GPU launch per run: the plain per-run GPU baseline.  The batched alternatives
are ``StatevectorSweep.fidelity_grad`` (adjoint, one launch for all angle
vectors and inputs) and ``batched_fd_fidelity_grad`` below (all perturbed
angle vectors in one forward launch).
"""
from __future__ import annotations

import numpy as np
import torch

__all__ = ["fd_gradient", "psr_gradient", "get_gradient", "fd_hessian", "psr_hessian", "get_hessian",
           "batched_fd_fidelity_grad"]


def fd_gradient(f, x, h=1e-5, type="central"):
    if type not in ("central", "forward", "backward"):
        raise UserWarning(f"Expected type to be 'central', 'forward', or 'backward' but {type} was given")
    x = np.asarray(x, dtype=float)
    n = len(x)
    grad = np.zeros(n)
    eye = np.eye(n)
    f0 = None if type == "central" else f(x)
    for i in range(n):
        if type == "central":
            grad[i] = (f(x + h * eye[i]) - f(x - h * eye[i])) / (2 * h)
        elif type == "forward":
            grad[i] = (f(x + h * eye[i]) - f0) / h
        else:
            grad[i] = (f0 - f(x - h * eye[i])) / h
    return grad


def psr_gradient(cost, x, shift=1.5):
    x = np.asarray(x, dtype=float)
    eye = np.eye(len(x))
    return np.array([(cost(x + shift * eye[i]) - cost(x - shift * eye[i])) / (2 * shift) for i in range(len(x))])


def get_gradient(cost, x, method="parameter-shift", *args, **kwargs):
    if method in ("parameter-shift", "psr", "parametershift"):
        return psr_gradient(cost, x, *args, **kwargs)
    if method in ("finite-differences", "fd", "finitedifferences"):
        return fd_gradient(cost, x, *args, **kwargs)
    raise UserWarning(
        f"Expected method to be 'parameter-shift' or 'finite-difference' but {method} was given"
    )


def _mixed_second(f, x, i, j, h, type):
    """One Hessian entry by second differences along e_i and e_j (the
    evaluation points and their arithmetic order of _finite_difference.py:28-55,
    so that the same cost gives the same entry)."""
    eye = np.eye(len(x))
    a, b = h * eye[i], h * eye[j]
    if type == "central":
        return (f(x + a + b) - f(x + a - b) - f(x - a + b) + f(x - a - b)) / (4 * h**2)
    if type == "forward":
        return (f(x + a + b) - f(x + a) - f(x + b) + f(x)) / h**2
    return (f(x) - f(x - a) - f(x - b) + f(x - a - b)) / h**2


def fd_hessian(f, x, h=1e-5, type="central"):
    """Hessian of a black-box cost by finite differences, every (i, j) entry
    from its own four evaluations (_finite_difference.py:28-55)."""
    if type not in ("central", "forward", "backward"):
        raise UserWarning(f"Expected type to be 'central', 'forward', or 'backward' but {type} was given")
    x = np.asarray(x, dtype=float)
    n = len(x)
    return np.array([[_mixed_second(f, x, i, j, h, type) for j in range(n)] for i in range(n)]).reshape(n, n)


def psr_hessian(cost, x, shift=1.5):
    """The reference's "parameter shift" Hessian: the central mixed difference
    with step ``shift`` (_parameter_shift.py:28-46)."""
    x = np.asarray(x, dtype=float)
    n = len(x)
    return np.array([[_mixed_second(cost, x, i, j, shift, "central") for j in range(n)]
                     for i in range(n)]).reshape(n, n)


def get_hessian(cost, x, method="parameter-shift", *args, **kwargs):
    if method in ("parameter-shift", "psr", "parametershift"):
        return psr_hessian(cost, x, *args, **kwargs)
    if method in ("finite-differences", "fd", "finitedifferences"):
        return fd_hessian(cost, x, *args, **kwargs)
    raise UserWarning(
        f"Expected method to be 'parameter-shift' or 'finite-difference' but {method} was given"
    )


def batched_fd_fidelity_grad(sweep, angles, inputs, targets, h=1e-4):
    """Central finite-difference gradient of 1 - mean_j |<t_j|z_j>|^2 with all
    2A perturbed angle vectors x J inputs evaluated in one forward launch per
    angle vector (device-side FD, for comparison with the adjoint)."""
    dev = sweep.device
    ang = torch.as_tensor(np.asarray(angles), dtype=torch.float64, device=dev).reshape(-1, sweep.n_angles)
    inp = torch.as_tensor(np.asarray(inputs), dtype=sweep.dtype, device=dev)
    tg = torch.as_tensor(np.asarray(targets), dtype=sweep.dtype, device=dev)
    V, A = ang.shape
    J = inp.shape[0]
    eye = torch.eye(A, dtype=torch.float64, device=dev) * h
    losses, grads = [], []
    for v in range(V):
        pert = torch.cat([ang[v] + eye, ang[v] - eye, ang[v : v + 1]], 0)  # [2A+1, A]
        P = pert.shape[0]
        out, _, _ = sweep.forward(pert.repeat_interleave(J, 0), inp.repeat(P, 1), ref_phase=False)
        f = (out.reshape(P, J, -1).conj() * tg.unsqueeze(0)).sum(-1).abs() ** 2
        loss = 1 - f.to(torch.float64).mean(1)
        grads.append((loss[:A] - loss[A : 2 * A]) / (2 * h))
        losses.append(loss[-1])
    return torch.stack(losses), torch.stack(grads)
