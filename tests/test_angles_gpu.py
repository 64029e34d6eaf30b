"""Angles far outside [0, 2pi), negative angles and angles after a training
run, through every kernel family against the complex128 oracle.  mentpy takes
double angles of any size (np_simulator_sv.py:246-249, ment.py:231-232);
the kernels reduce them without first rounding the double to float, so the
error must not grow with |theta|."""
import numpy as np
import pytest
import torch

from helpers import exec_plan_sv_adjoint, haar_states
from mentpy_gb300 import circuit as C
from mentpy_gb300.dm import DensityMatrixSweep
from mentpy_gb300.plan import compile_plan
from mentpy_gb300.sweep import STREAMED, StatevectorSweep
from oracle import gradients as G
from oracle import sweep as oracle

pytestmark = pytest.mark.gpu

TOL_INFID_C64 = 1e-5
TOL_AMP_C64 = 2e-5
TOL_RHO_C64 = 2e-5
TOL_GRAD_C64 = 2e-4

RANGES = {"small": (0.0, 2 * np.pi), "1e2": (-1e2, 1e2), "1e4": (-1e4, 1e4), "neg": (-3e3, 0.0),
          "1e6": (-1e6, 1e6)}


def _infid(a, b):
    a = np.asarray(a, dtype=np.complex128)
    a = a / np.linalg.norm(a, axis=-1, keepdims=True)
    b = b / np.linalg.norm(b, axis=-1, keepdims=True)
    return 1.0 - np.abs(np.sum(a.conj() * b, axis=-1)) ** 2


@pytest.mark.parametrize("rng_name", sorted(RANGES))
def test_register_kernel_any_magnitude(rng_name):
    lo, hi = RANGES[rng_name]
    circ = C.many_wires([8] * 4)
    rng = np.random.default_rng(101)
    B = 512
    ang = rng.uniform(lo, hi, size=(B, len(circ.trainable_nodes)))
    psi = haar_states(rng, 4, B)
    out, st, _ = StatevectorSweep(circ).forward(ang, psi)
    assert (st.cpu().numpy() == 0).all()
    ref, _ = oracle.run_sv_batch(circ, ang, psi)
    out = out.cpu().numpy()
    assert _infid(out, ref).max() < TOL_INFID_C64
    assert np.abs(out - ref).max() < TOL_AMP_C64, rng_name


def test_fp64_check_mode_large_angles():
    circ = C.grid_cluster(3, 5)
    rng = np.random.default_rng(102)
    B = 64
    ang = rng.uniform(-1e4, 1e4, size=(B, len(circ.trainable_nodes)))
    psi = haar_states(rng, 3, B)
    out, st, _ = StatevectorSweep(circ, dtype=torch.complex128).forward(ang, psi)
    ref, _ = oracle.run_sv_batch(circ, ang, psi)
    out = out.cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    assert _infid(out, ref).max() < 1e-12
    assert np.abs(out - ref).max() < 1e-10


@pytest.mark.parametrize("rows,cols", [(9, 4), (12, 3)])
def test_streamed_kernel_large_angles(rows, cols):
    circ = C.grid_cluster(rows, cols)
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(103)
    B = 4
    ang = rng.uniform(-1e4, 1e4, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    out, st, _ = sw.forward(ang, psi, variant=STREAMED)
    assert (st.cpu().numpy() == 0).all()
    ref, _ = oracle.run_sv_batch(circ, ang, psi)
    out = out.cpu().numpy()
    assert _infid(out, ref).max() < TOL_INFID_C64
    assert np.abs(out - ref).max() < TOL_AMP_C64


def test_adjoint_large_angles():
    circ = C.many_wires([6] * 3)
    plan = compile_plan(circ, "sv")
    rng = np.random.default_rng(104)
    R = 4
    ang = rng.uniform(-1e4, 1e4, size=(R, plan.n_angles))
    psi = haar_states(rng, plan.n_in, R)
    g = rng.standard_normal((R, 2**plan.n_out)) + 1j * rng.standard_normal((R, 2**plan.n_out))
    sw = StatevectorSweep(plan=plan)
    grad = sw.adjoint(ang, psi, g).cpu().numpy()
    for r in range(R):
        ref = G.linear_functional_grad(circ, ang[r], psi[r], g[r], h=1e-5)
        assert np.abs(grad[r] - ref).max() / (1 + np.abs(ref).max()) < TOL_GRAD_C64
        exact = exec_plan_sv_adjoint(plan, ang[r], psi[r], g[r])
        assert np.abs(grad[r] - exact).max() / (1 + np.abs(exact).max()) < TOL_GRAD_C64
    # the fused fidelity gradient
    J = 5
    inp = haar_states(rng, plan.n_in, J)
    tg = haar_states(rng, plan.n_out, J)
    loss, fg = sw.fidelity_grad(ang[:2], inp, tg)
    for v in range(2):
        assert abs(float(loss[v]) - G.fidelity_loss(circ, ang[v], inp, tg)) < 1e-5
        ref = G.fidelity_grad_fd(circ, ang[v], inp, tg, h=1e-4)
        assert np.abs(fg[v].cpu().numpy() - ref).max() < TOL_GRAD_C64


@pytest.mark.parametrize("noise", [0.0, 0.01])
def test_density_matrix_large_angles(noise):
    circ = C.many_wires([6] * 5)  # window 6
    sw = DensityMatrixSweep(circ)
    rng = np.random.default_rng(105)
    B = 64
    ang = rng.uniform(-1e4, 1e4, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    rho, outc, st, _ = sw.forward(ang, psi, noise=noise)
    assert (st.cpu().numpy() == 0).all()
    ref, ref_out, _ = oracle.run_dm_batch(circ, ang, psi, noise_p=noise)
    assert np.abs(rho.cpu().numpy() - ref).max() < TOL_RHO_C64
    assert np.array_equal(outc.cpu().numpy(), ref_out)


def test_density_matrix_adjoint_large_angles():
    circ = C.many_wires([5] * 3)
    sw = DensityMatrixSweep(circ)
    rng = np.random.default_rng(106)
    R = 3
    ang = rng.uniform(-1e4, 1e4, size=(R, sw.n_angles))
    psi = haar_states(rng, sw.n_in, R)
    d = 2**sw.n_out
    gam = rng.standard_normal((R, d, d)) + 1j * rng.standard_normal((R, d, d))
    gam = gam + gam.conj().transpose(0, 2, 1)
    grad, _, st = sw.adjoint(ang, psi, gam, noise=0.01)
    assert (st.cpu().numpy() == 0).all()
    for r in range(R):
        ref = G.dm_linear_functional_grad(circ, ang[r], psi[r], gam[r], noise_p=0.01, h=1e-5)
        assert np.abs(grad[r].cpu().numpy() - ref).max() / (1 + np.abs(ref).max()) < TOL_GRAD_C64


def test_angles_after_a_training_run():
    """Angles after 500 Adam iterations (started far outside [0, 2pi)): the
    sweep at the trained angles still matches the oracle."""
    from mentpy_gb300.train import FidelityTrainer

    circ = C.many_wires([5] * 3)
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(107)
    V, J = 64, 8
    x0 = rng.uniform(-50, 50, size=(V, sw.n_angles))
    inp = haar_states(rng, 3, J)
    tg = haar_states(rng, 3, J)
    tr = FidelityTrainer(sw, inp, tg, x0, step_size=0.5)
    ang = tr.run(500).cpu().numpy()
    assert np.abs(ang - x0).max() > 1.0  # the optimiser moved them
    out, st, _ = sw.forward(ang, np.tile(inp[:1], (V, 1)))
    ref, _ = oracle.run_sv_batch(circ, ang, inp[:1])
    out = out.cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    assert _infid(out, ref).max() < TOL_INFID_C64
    assert np.abs(out - ref).max() < TOL_AMP_C64
