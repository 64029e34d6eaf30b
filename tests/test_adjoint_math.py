"""The adjoint recurrences the GPU kernels implement, checked in complex128
against central finite differences of the oracle (no GPU)."""
import numpy as np
import pytest

from helpers import circuit_from_spec, exec_plan_sv, exec_plan_sv_adjoint, load_golden
from mentpy_gb300.plan import compile_plan
from oracle import gradients as G


@pytest.mark.parametrize("name", ["lin9_haar", "grid3x4_w6", "lin7_fixed", "rand_muta21_1_w5_xx",
                                  "rand_grid2x5_w5", "lin6_w4"])
def test_adjoint_recurrence_matches_fd(name):
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    kw = spec["sim_kwargs"]
    plan = compile_plan(circ, "sv", **kw)
    rng = np.random.default_rng(5)
    for r in range(len(data["angles"])):
        ang = data["angles"][r]
        psi = data["inputs"][r] if "inputs" in data else np.ones(2**plan.n_in) / np.sqrt(2**plan.n_in)
        g = rng.standard_normal(2**plan.n_out) + 1j * rng.standard_normal(2**plan.n_out)
        adj = exec_plan_sv_adjoint(plan, ang, psi, g)
        fd = G.linear_functional_grad(circ, ang, psi, g, **kw)
        assert np.abs(adj - fd).max() < 1e-7 * (1 + np.abs(fd).max())


def test_canonical_output_is_plan_output_without_phase():
    spec, data = load_golden("grid3x5")
    circ = circuit_from_spec(spec)
    plan = compile_plan(circ, "sv")
    for r in range(3):
        z = exec_plan_sv(plan, data["angles"][r], data["inputs"][r], ref_phase=False)
        assert np.allclose(z, G.canonical_sv(circ, data["angles"][r], data["inputs"][r]), atol=1e-12)


def test_fidelity_grad_seed():
    # the fused fidelity seed: grad_out = -(2/J) <t|z> t per run
    spec, data = load_golden("lin9_haar")
    circ = circuit_from_spec(spec)
    plan = compile_plan(circ, "sv")
    rng = np.random.default_rng(9)
    ang = data["angles"][0]
    inputs = data["inputs"]
    targets = rng.standard_normal((4, 2)) + 1j * rng.standard_normal((4, 2))
    targets /= np.linalg.norm(targets, axis=1, keepdims=True)
    J = len(inputs)
    total = np.zeros(plan.n_angles)
    for j in range(J):
        z = exec_plan_sv(plan, ang, inputs[j], ref_phase=False)
        a = np.vdot(targets[j], z)
        total += exec_plan_sv_adjoint(plan, ang, inputs[j], -(2.0 / J) * a * targets[j])
    fd = G.fidelity_grad(circ, ang, inputs, targets)
    assert np.abs(total - fd).max() < 1e-7


def _coef_gen(plane, theta):
    """(amp, c, damp, dc) of a step of plane code ``plane`` (0 XY, 1 X, 2 Y,
    3 XZ, 4 YZ): phi = amp psi0 + c psi1 and the angle derivatives the
    block-per-run adjoint uses (csrc/sv_adj_wide.cu)."""
    if plane in (0, 1, 2):
        c = np.exp(-1j * {0: theta, 1: 0.0, 2: np.pi / 2}[plane])
        return 1.0, c, 0.0, (-1j * c if plane == 0 else 0.0)
    h = np.angle(np.exp(1j * theta)) / 2
    amp, d = np.cos(h) + np.sin(h), np.cos(h) - np.sin(h)
    sg = -1.0 if amp < 0 else 1.0
    amp, d = sg * amp, sg * d
    if plane == 3:
        return amp, d + 0j, 0.5 * d, -0.5 * amp + 0j
    return amp, -1j * d, 0.5 * d, 0.5j * amp


def _exec_plan_sv_adjoint_wide(plan, angles, psi_in, grad_out, scale=True):
    """The block-per-run adjoint's chain in complex128: every step first
    scales the window by an exact power of two alpha_k (its squared norm into
    [1, 4)), the history keeps the unscaled pre-step halves, and the backward
    step carries alpha_k into the gradient term and into lambda."""
    from helpers import DEAD, _initial_window, _out_index, _popc

    w = plan.window
    idx = np.arange(2**w)
    psi = _initial_window(plan, psi_in).astype(complex)
    steps = []
    nrm = float(np.vdot(psi, psi).real)
    for k in range(plan.n_steps):
        e = (np.frexp(nrm)[1] - 1) >> 1 if scale else 0
        al = 2.0 ** (-e)
        p = k % w
        a = int(plan.step_angle[k])
        theta = angles[a] if a >= 0 else plan.step_fixed_angle[k]
        amp, c, damp, dc = _coef_gen(int(plan.step_plane[k]), theta)
        lo = idx[((idx >> p) & 1) == 0]
        hi = lo | (1 << p)
        steps.append((al, amp, c, damp, dc, psi[lo].copy(), psi[hi].copy()))
        phi = al * (amp * psi[lo] + c * psi[hi])
        m = int(plan.step_mask[k])
        psi = psi.copy()
        psi[lo] = phi
        psi[hi] = 0 if (m & DEAD) else phi * np.where(_popc(hi & m) & 1, -1.0, 1.0)
        nrm = float(np.vdot(psi, psi).real)
    oi = _out_index(plan)
    n = np.linalg.norm(psi)
    g = np.asarray(grad_out, complex)
    lam = np.zeros_like(psi)
    lam[oi] = (g - np.real(np.vdot(psi[oi], g)) / n**2 * psi[oi]) / n
    grad = np.zeros(plan.n_angles)
    for k in range(plan.n_steps - 1, -1, -1):
        al, amp, c, damp, dc, u0, u1 = steps[k]
        p = k % w
        lo = idx[((idx >> p) & 1) == 0]
        hi = lo | (1 << p)
        m = int(plan.step_mask[k])
        mu = lam[lo] if (m & DEAD) else lam[lo] + np.where(_popc(hi & m) & 1, -1.0, 1.0) * lam[hi]
        a = int(plan.step_angle[k])
        if a >= 0:
            grad[a] += al * np.real(damp * np.sum(np.conj(mu) * u0) + dc * np.sum(np.conj(mu) * u1))
        lam = lam.copy()
        lam[lo] = al * amp * mu
        lam[hi] = al * np.conj(c) * mu
    return grad


@pytest.mark.parametrize("planes", [{}, {1: "XZ"}, {2: "YZ"}, {1: "XZ", 2: "YZ", 4: "XZ"}, {0: "YZ", 3: "XZ"}])
def test_block_adjoint_chain_matches_fd(planes):
    """The block-per-run adjoint's chain (power-of-two scaling, XY / XZ / YZ
    derivatives) against central differences of the oracle, with normalised
    and unnormalised inputs, and the scaling neutral to rounding."""
    from mentpy_gb300 import circuit as C

    circ = C.linear_cluster(8)
    for node, pl in planes.items():
        circ[node] = C.Ment(pl)
    plan = compile_plan(circ, "sv", extended_planes=True)
    rng = np.random.default_rng(17)
    for scale_in in (1.0, 3e-7, 5e6):
        ang = rng.uniform(-7, 7, size=plan.n_angles)
        psi = rng.standard_normal(2) + 1j * rng.standard_normal(2)
        psi = scale_in * psi / np.linalg.norm(psi)
        g = rng.standard_normal(2**plan.n_out) + 1j * rng.standard_normal(2**plan.n_out)
        adj = _exec_plan_sv_adjoint_wide(plan, ang, psi, g)
        fd = G.linear_functional_grad(circ, ang, psi, g)
        assert np.abs(adj - fd).max() < 1e-7 * (1 + np.abs(fd).max()), (planes, scale_in)
        plain = _exec_plan_sv_adjoint_wide(plan, ang, psi, g, scale=False)
        assert np.abs(adj - plain).max() < 1e-12 * (1 + np.abs(plain).max())


@pytest.mark.parametrize("name", ["lin9_haar", "grid3x4_w6", "rand_grid2x5_w5"])
def test_block_adjoint_chain_is_the_register_chain(name):
    """On XY-plane reference fixtures the block-per-run chain gives the
    register kernels' gradient."""
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    kw = spec["sim_kwargs"]
    plan = compile_plan(circ, "sv", **kw)
    rng = np.random.default_rng(6)
    for r in range(min(3, len(data["angles"]))):
        ang = data["angles"][r]
        psi = data["inputs"][r] if "inputs" in data else np.ones(2**plan.n_in) / np.sqrt(2**plan.n_in)
        g = rng.standard_normal(2**plan.n_out) + 1j * rng.standard_normal(2**plan.n_out)
        a1 = _exec_plan_sv_adjoint_wide(plan, ang, psi, g)
        a2 = exec_plan_sv_adjoint(plan, ang, psi, g)
        assert np.abs(a1 - a2).max() < 1e-10 * (1 + np.abs(a2).max())
