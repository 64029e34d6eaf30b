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
