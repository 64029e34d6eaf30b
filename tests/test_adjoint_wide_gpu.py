"""Adjoint kernel for windows 9..20 (a block per run, per-step history in the
workspace): gradients against complex128 central differences of the oracle
(h = 1e-4, the finite-difference step of mentpy's fd_gradient use), the fused
fidelity loss, and the streamed-window grid of 16 x 10 (w = 17) through a
directional derivative."""
import numpy as np
import pytest
import torch

from helpers import haar_states
from mentpy_gb300 import circuit as C
from mentpy_gb300.sweep import StatevectorSweep
from oracle import gradients as G

pytestmark = pytest.mark.gpu

TOL_GRAD_C64 = 2e-4

WIDE = {"mw4x8_w9": lambda: C.many_wires([4] * 8), "mw3x9_w10": lambda: C.many_wires([3] * 9),
        "mw3x11_w12": lambda: C.many_wires([3] * 11), "mw3x14_w15": lambda: C.many_wires([3] * 14),
        "mw3x16_w17": lambda: C.many_wires([3] * 16)}


def _grad_out(rng, B, n_out):
    return rng.standard_normal((B, 2**n_out)) + 1j * rng.standard_normal((B, 2**n_out))


@pytest.mark.parametrize("name", sorted(WIDE))
def test_wide_generic_adjoint_matches_fd(name):
    circ = WIDE[name]()
    sw = StatevectorSweep(circ)
    assert sw.plan.window > 8
    rng = np.random.default_rng(201)
    B = 1 if sw.plan.window > 16 else 2
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    inp = haar_states(rng, sw.n_in, B)
    g = _grad_out(rng, B, sw.n_out)
    st = torch.empty(B, dtype=torch.int32, device="cuda")
    grad = sw.adjoint(ang, inp, g, status=st).cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    for r in range(B):
        ref = G.linear_functional_grad(circ, ang[r], inp[r], g[r], h=1e-4)
        err = np.abs(grad[r] - ref).max() / (1 + np.abs(ref).max())
        assert err < TOL_GRAD_C64, (name, r, err)


def test_wide_fidelity_grad_matches_oracle():
    circ = C.many_wires([3] * 11)  # w = 12, 22 angles
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(202)
    V, J = 2, 3
    ang = rng.uniform(0, 2 * np.pi, size=(V, sw.n_angles))
    inputs = haar_states(rng, sw.n_in, J)
    targets = haar_states(rng, sw.n_out, J)
    loss, grad = sw.fidelity_grad(ang, inputs, targets)
    loss, grad = loss.cpu().numpy(), grad.cpu().numpy()
    for v in range(V):
        assert abs(loss[v] - G.fidelity_loss(circ, ang[v], inputs, targets)) < 1e-5
        ref = G.fidelity_grad(circ, ang[v], inputs, targets, h=1e-4)
        assert np.abs(grad[v] - ref).max() < TOL_GRAD_C64, (v, np.abs(grad[v] - ref).max())


def test_grid16x10_directional_derivative():
    """The streamed workload's circuit (w = 17, 144 angles, 144 steps): the
    adjoint's gradient along random directions against the oracle's central
    difference of the same linear functional."""
    circ = C.grid_cluster(16, 10)
    sw = StatevectorSweep(circ)
    assert sw.plan.window == 17
    rng = np.random.default_rng(203)
    B = 2
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    inp = haar_states(rng, sw.n_in, B)
    g = _grad_out(rng, B, sw.n_out)
    st = torch.empty(B, dtype=torch.int32, device="cuda")
    grad = sw.adjoint(ang, inp, g, status=st).cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    h = 1e-4
    for r in range(B):
        d = rng.standard_normal(sw.n_angles)
        d /= np.linalg.norm(d)
        f = lambda a: float(np.real(np.vdot(g[r], G.canonical_sv(circ, a, inp[r]))))  # noqa: E731
        fd = (f(ang[r] + h * d) - f(ang[r] - h * d)) / (2 * h)
        got = float(grad[r] @ d)
        assert abs(got - fd) < TOL_GRAD_C64 * (1 + np.abs(grad[r]).max()), (r, got, fd)


def test_wide_adjoint_persistent_loop_is_deterministic():
    """More runs than resident blocks (w = 15: a 1024-thread block per run):
    each block loops over runs, and a run's gradient does not depend on the
    slot it ran in; a batch of five runs shares each run among a cluster of
    four blocks (other partial-sum order: equal to float rounding)."""
    circ = C.many_wires([3] * 14)
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(204)
    B = 700
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    inp = haar_states(rng, sw.n_in, B)
    g = _grad_out(rng, B, sw.n_out)
    st = torch.empty(B, dtype=torch.int32, device="cuda")
    grad = sw.adjoint(ang, inp, g, status=st)
    part = sw.adjoint(ang[-5:], inp[-5:], g[-5:])
    torch.cuda.synchronize()
    assert (st.cpu().numpy() == 0).all()
    g_last = grad[-5:].cpu().numpy()
    assert np.abs(g_last - part.cpu().numpy()).max() < 1e-5 * (1 + np.abs(g_last).max())
    # two launches of the same batch: the same bits
    again = sw.adjoint(ang[-5:], inp[-5:], g[-5:])
    assert torch.equal(part, again)
    ref = G.linear_functional_grad(circ, ang[B - 1], inp[B - 1], g[B - 1], h=1e-4)
    assert np.abs(grad[-1].cpu().numpy() - ref).max() / (1 + np.abs(ref).max()) < TOL_GRAD_C64
