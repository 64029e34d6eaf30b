"""Density-matrix adjoint through the noisy channel, against complex128 finite
differences of the oracle; autograd wrapper; uneven multi-circuit batch."""
import numpy as np
import pytest
import torch

from helpers import circuit_from_spec, haar_states, load_golden
from mentpy_gb300 import circuit as C
from mentpy_gb300.dm import DensityMatrixSweep, UnevenDensityMatrixBatch, dm_states
from mentpy_gb300.plan import compile_plan
from oracle import gradients as G

pytestmark = pytest.mark.gpu

TOL_GRAD_C64 = 2e-4  # relative to 1 + max |grad|


def _herm(rng, d):
    g = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    return g + g.conj().T


@pytest.mark.parametrize("build", [lambda: C.linear_cluster(5), lambda: C.many_wires([4] * 3),
                                   lambda: C.grid_cluster(3, 3), lambda: C.many_wires([5] * 6),
                                   lambda: C.grid_cluster(2, 5)])
@pytest.mark.parametrize("p", [0.0, 0.05])
def test_dm_adjoint_matches_fd(build, p):
    circ = build()
    sw = DensityMatrixSweep(circ)
    rng = np.random.default_rng(44)
    B = 3
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    d = 2**sw.n_out
    gam = np.stack([_herm(rng, d) for _ in range(B)])
    grad, rho, st = sw.adjoint(ang, psi, gam, noise=p)
    assert (st.cpu().numpy() == 0).all()
    grad = grad.cpu().numpy()
    rho_f, _, _, _ = sw.forward(ang, psi, noise=p)
    assert (rho - rho_f).abs().max().item() < 1e-6
    for r in range(B):
        ref = G.dm_linear_functional_grad(circ, ang[r], psi[r], gam[r], noise_p=p)
        err = np.abs(grad[r] - ref).max() / (1 + np.abs(ref).max())
        assert err < TOL_GRAD_C64, (r, err)


@pytest.mark.parametrize("name", ["dm_planes_lin5", "dm_threshold_lin4_w1", "dm_scaled_input_lin5", "lin7_fixed"])
def test_dm_adjoint_reference_cases(name):
    # XZ/YZ planes, outcome-1 steps (prob0 < 1e-4), unnormalised inputs, fixed angles
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    kw = spec["sim_kwargs"]
    sw = DensityMatrixSweep(circ, **kw)
    rng = np.random.default_rng(5)
    R = len(data["angles"])
    d = 2**sw.n_out
    gam = np.stack([_herm(rng, d) for _ in range(R)])
    inputs = data.get("inputs")
    grad, _, st = sw.adjoint(data["angles"], inputs, gam)
    grad = grad.cpu().numpy()
    for r in range(R):
        psi = None if inputs is None else inputs[r]
        ref = G.dm_linear_functional_grad(circ, data["angles"][r], psi, gam[r], h=1e-6, **kw)
        err = np.abs(grad[r] - ref).max() / (1 + np.abs(ref).max())
        assert err < TOL_GRAD_C64, (name, r, err)


def test_dm_autograd_fidelity():
    circ = C.grid_cluster(3, 3)
    sw = DensityMatrixSweep(circ)
    rng = np.random.default_rng(6)
    B = 4
    ang0 = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, 3, B)
    tgt = haar_states(rng, 3, B)
    a = torch.tensor(ang0, device="cuda", requires_grad=True)
    rho = dm_states(sw, a, torch.as_tensor(psi, dtype=torch.complex64, device="cuda"), noise=0.02)
    t = torch.as_tensor(tgt, dtype=torch.complex64, device="cuda")
    fid = torch.einsum("bi,bij,bj->b", t.conj(), rho, t).real
    (1 - fid.to(torch.float64)).sum().backward()
    for r in range(B):
        def loss(x):
            from oracle import sweep as S

            rr, _, _ = S.run_dm(circ, x, psi[r], noise_p=0.02)
            return 1 - float(np.real(np.vdot(tgt[r], rr @ tgt[r])))

        ref = G.central_fd(loss, ang0[r])
        assert np.abs(a.grad[r].cpu().numpy() - ref).max() < TOL_GRAD_C64


def test_uneven_adjoint_matches_single_circuit():
    rng = np.random.default_rng(9)
    circs = [C.many_wires([int(rng.integers(4, 9))] * int(rng.integers(2, 7))) for _ in range(12)]
    plans = [compile_plan(c, "dm") for c in circs]
    ub = UnevenDensityMatrixBatch(plans)
    buf = ub.allocate()
    buf["grad_out"] = torch.zeros((len(plans), 4**ub.max_out), dtype=torch.complex64, device="cuda")
    gams = []
    for c, p in enumerate(plans):
        buf["angles"][c, : p.n_angles] = torch.as_tensor(rng.uniform(0, 2 * np.pi, p.n_angles))
        buf["inputs"][c, : 2**p.n_in] = torch.as_tensor(haar_states(rng, p.n_in, 1)[0], dtype=torch.complex64)
        g = _herm(rng, 2**p.n_out)
        gams.append(g)
        buf["grad_out"][c, : g.size] = torch.as_tensor(g.reshape(-1), dtype=torch.complex64)
    ub.adjoint(buf, noise=0.01)
    torch.cuda.synchronize()
    assert (buf["status"] == 0).all()
    for c, p in enumerate(plans):
        sw = DensityMatrixSweep(plan=p)
        g1, _, _ = sw.adjoint(buf["angles"][c : c + 1, : p.n_angles], buf["inputs"][c : c + 1, : 2**p.n_in],
                              gams[c][None], noise=0.01)
        assert (buf["grad"][c, : p.n_angles] - g1[0]).abs().max().item() < 1e-9


@pytest.mark.parametrize("wires,p", [(7, 0.0), (7, 0.05), (8, 0.05)])
def test_dm_adjoint_workspace_windows_match_fd(wires, p):
    """Windows 8 and 9: the matrix in a workspace slot, a 1024-thread block
    per run."""
    circ = C.many_wires([3] * wires)
    sw = DensityMatrixSweep(circ)
    assert sw.plan.window == wires + 1
    rng = np.random.default_rng(45 + wires)
    B = 2 if wires == 7 else 1
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    d = 2**sw.n_out
    gam = np.stack([_herm(rng, d) for _ in range(B)])
    grad, rho, st = sw.adjoint(ang, psi, gam, noise=p)
    assert (st.cpu().numpy() == 0).all()
    grad = grad.cpu().numpy()
    rho_f, _, _, _ = sw.forward(ang, psi, noise=p)
    assert (rho - rho_f).abs().max().item() < 1e-6
    for r in range(B):
        ref = G.dm_linear_functional_grad(circ, ang[r], psi[r], gam[r], noise_p=p)
        err = np.abs(grad[r] - ref).max() / (1 + np.abs(ref).max())
        assert err < TOL_GRAD_C64, (r, err)


def test_dm_adjoint_window10_directional_derivative():
    from oracle import sweep as O

    circ = C.many_wires([3] * 9)
    sw = DensityMatrixSweep(circ)
    assert sw.plan.window == 10
    rng = np.random.default_rng(49)
    ang = rng.uniform(0, 2 * np.pi, size=(1, sw.n_angles))
    psi = haar_states(rng, sw.n_in, 1)
    gam = _herm(rng, 2**sw.n_out)[None]
    grad, _, st = sw.adjoint(ang, psi, gam, noise=0.02)
    assert int(st[0]) == 0
    dvec = rng.standard_normal(sw.n_angles)
    dvec /= np.linalg.norm(dvec)
    h = 1e-4

    def f(a):
        rho, _, _ = O.run_dm(circ, a, psi[0], noise_p=0.02)
        return float(np.real(np.vdot(gam[0], rho)))

    fd = (f(ang[0] + h * dvec) - f(ang[0] - h * dvec)) / (2 * h)
    got = float(grad[0].cpu().numpy() @ dvec)
    assert abs(got - fd) < TOL_GRAD_C64 * (1 + np.abs(grad[0].cpu().numpy()).max()), (got, fd)


def test_dm_adjoint_workspace_window_more_runs_than_slots():
    """Window 8 with more runs than resident 1024-thread blocks: blocks loop
    over runs, and a run's gradient does not depend on its slot."""
    circ = C.many_wires([3] * 7)
    sw = DensityMatrixSweep(circ)
    rng = np.random.default_rng(50)
    B = 400
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    d = 2**sw.n_out
    gam = np.stack([_herm(rng, d) for _ in range(B)])
    grad, _, st = sw.adjoint(ang, psi, gam, noise=0.01)
    part, _, _ = sw.adjoint(ang[-3:], psi[-3:], gam[-3:], noise=0.01)
    assert (st.cpu().numpy() == 0).all()
    assert torch.equal(grad[-3:], part)
