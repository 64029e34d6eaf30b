"""Adjoint kernels: gradients against complex128 finite differences of the oracle,
the fused fidelity loss, and the autograd.Function."""
import numpy as np
import pytest
import torch

from helpers import circuit_from_spec, exec_plan_sv_adjoint, haar_states, load_golden
from mentpy_gb300 import circuit as C
from mentpy_gb300.autograd import sweep_states
from mentpy_gb300.gradients import batched_fd_fidelity_grad
from mentpy_gb300.plan import compile_plan
from mentpy_gb300.sweep import StatevectorSweep
from oracle import gradients as G

pytestmark = pytest.mark.gpu

# complex64 amplitudes, FP64 reductions: gradient error vs the complex128 reference
TOL_GRAD_C64 = 2e-4
TOL_GRAD_F64 = 1e-9

CASES = ["lin9_haar", "mw4x8", "mw6x12", "grid3x4_w6", "lin7_fixed", "lin6_w4",
         "rand_muta21_1_w5_xx", "rand_grid2x5_w5", "teleport_lin5"]


def _case(name):
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    kw = spec["sim_kwargs"]
    plan = compile_plan(circ, "sv", **kw)
    n = plan.n_in
    inputs = data["inputs"] if "inputs" in data else np.tile(np.ones(2**n) / np.sqrt(2**n), (len(data["angles"]), 1))
    return circ, kw, plan, data["angles"], inputs


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_generic_adjoint_matches_fd(name, dtype):
    circ, kw, plan, angles, inputs = _case(name)
    rng = np.random.default_rng(17)
    R = len(angles)
    g = rng.standard_normal((R, 2**plan.n_out)) + 1j * rng.standard_normal((R, 2**plan.n_out))
    sw = StatevectorSweep(plan=plan, dtype=dtype)
    st = torch.empty(R, dtype=torch.int32, device="cuda")
    grad = sw.adjoint(angles, inputs, g, status=st).cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    for r in range(R):
        ref = G.linear_functional_grad(circ, angles[r], inputs[r], g[r], h=1e-5, **kw)
        err = np.abs(grad[r] - ref).max() / (1 + np.abs(ref).max())
        # central FD at h=1e-5 is itself accurate to ~1e-8
        assert err < (TOL_GRAD_C64 if dtype == torch.complex64 else 1e-7), (name, r, err)
        if dtype == torch.complex128:
            exact = exec_plan_sv_adjoint(plan, angles[r], inputs[r], g[r])
            err = np.abs(grad[r] - exact).max() / (1 + np.abs(exact).max())
            assert err < TOL_GRAD_F64, (name, r, err)


def test_fixed_angle_nodes_get_zero_gradient():
    circ, kw, plan, angles, inputs = _case("lin7_fixed")
    sw = StatevectorSweep(plan=plan)
    g = np.ones((len(angles), 2), complex)
    grad = sw.adjoint(angles, inputs, g).cpu().numpy()
    assert grad.shape == (len(angles), plan.n_angles)  # only trainable angles appear


@pytest.mark.parametrize("name,V,J", [("mw4x8", 3, 6), ("mw6x12", 2, 4), ("grid6x4", 2, 3)])
def test_fidelity_grad_matches_oracle(name, V, J):
    circ, kw, plan, _, _ = _case(name)
    rng = np.random.default_rng(23)
    A = plan.n_angles
    angles = rng.uniform(0, 2 * np.pi, size=(V, A))
    inputs = haar_states(rng, plan.n_in, J)
    targets = haar_states(rng, plan.n_out, J)
    sw = StatevectorSweep(plan=plan)
    loss, grad = sw.fidelity_grad(angles, inputs, targets)
    loss, grad = loss.cpu().numpy(), grad.cpu().numpy()
    for v in range(V):
        ref_loss = G.fidelity_loss(circ, angles[v], inputs, targets, **kw)
        assert abs(loss[v] - ref_loss) < 1e-5
        ref = G.fidelity_grad(circ, angles[v], inputs, targets, h=1e-5, **kw)
        assert np.abs(grad[v] - ref).max() < TOL_GRAD_C64, (v, np.abs(grad[v] - ref).max())


def test_fidelity_grad_matches_batched_fd_and_autograd():
    circ = C.many_wires([6] * 3)
    plan = compile_plan(circ, "sv")
    rng = np.random.default_rng(31)
    V, J = 2, 5
    angles = rng.uniform(0, 2 * np.pi, size=(V, plan.n_angles))
    inputs = haar_states(rng, 3, J)
    targets = haar_states(rng, 3, J)
    sw = StatevectorSweep(plan=plan)
    loss, grad = sw.fidelity_grad(angles, inputs, targets)
    fd_loss, fd_grad = batched_fd_fidelity_grad(sw, angles, inputs, targets, h=1e-3)
    assert torch.allclose(loss, fd_loss, atol=1e-5)
    assert (grad - fd_grad).abs().max() < 2e-3  # complex64 FD at h=1e-3
    # autograd through the differentiable sweep gives the same gradient
    a = torch.tensor(angles, dtype=torch.float64, device="cuda", requires_grad=True)
    inp = torch.as_tensor(inputs, dtype=torch.complex64, device="cuda")
    tg = torch.as_tensor(targets, dtype=torch.complex64, device="cuda")
    z = sweep_states(sw, a.repeat_interleave(J, 0), inp.repeat(V, 1))
    f = ((z.conj() * tg.repeat(V, 1)).sum(-1).abs() ** 2).reshape(V, J)
    L = (1 - f.to(torch.float64).mean(1)).sum()
    L.backward()
    assert (a.grad - grad).abs().max() < 1e-4


def test_fidelity_grad_large_batch_consistency():
    # many angle vectors in one launch; spot-check against single-vector launches
    circ = C.many_wires([12] * 6)
    plan = compile_plan(circ, "sv")
    rng = np.random.default_rng(41)
    V, J = 64, 32
    angles = rng.uniform(0, 2 * np.pi, size=(V, plan.n_angles))
    inputs = haar_states(rng, 6, J)
    targets = haar_states(rng, 6, J)
    sw = StatevectorSweep(plan=plan)
    loss, grad = sw.fidelity_grad(angles, inputs, targets)
    for v in (0, 17, 63):
        l1, g1 = sw.fidelity_grad(angles[v : v + 1], inputs, targets)
        assert abs(float(l1[0]) - float(loss[v])) < 1e-9
        assert (g1[0] - grad[v]).abs().max() < 1e-9
