"""The factored density-matrix recurrence (csrc/dm_fact.cuh) restated in
complex128 reproduces the reference fixtures and the full-matrix plan
executor, with noise and with outcome-1 steps (no GPU)."""
import numpy as np
import pytest

from helpers import circuit_from_spec, exec_plan_dm, exec_plan_dm_factored, golden_names, haar_states, load_golden
from mentpy_gb300 import circuit as C
from mentpy_gb300.plan import DEAD, compile_plan

DM_CASES = [n for n in golden_names() if "dm_rho" in load_golden(n)[1] and "dm_zexp_outcomes" not in load_golden(n)[1]]


@pytest.mark.parametrize("name", DM_CASES)
def test_factored_recurrence_matches_reference(name):
    spec, data = load_golden(name)
    plan = compile_plan(circuit_from_spec(spec), "dm", **spec["sim_kwargs"])
    if plan.window < 2 or not (int(plan.step_mask[-1]) & DEAD):
        pytest.skip("the factored kernel needs window >= 2 and a shrinking last step")
    n_in = len(spec["input_nodes"])
    for r in range(len(data["angles"])):
        psi = data["inputs"][r] if "inputs" in data else np.ones(2**n_in) / np.sqrt(2**n_in)
        rho, outc, _ = exec_plan_dm_factored(plan, data["angles"][r], psi)
        assert np.allclose(rho, data["dm_rho"][r], atol=1e-10), name
        assert outc == list(data["dm_outcomes"][r][: len(outc)])


@pytest.mark.parametrize("build", [lambda: C.many_wires([6] * 3), lambda: C.grid_cluster(3, 4),
                                   lambda: C.many_wires([5] * 6), lambda: C.grid_cluster(4, 3),
                                   lambda: C.many_wires([4] * 7)])
@pytest.mark.parametrize("p", [0.0, 0.05])
def test_factored_recurrence_matches_full_matrix(build, p):
    circ = build()
    plan = compile_plan(circ, "dm")
    rng = np.random.default_rng(9)
    for _ in range(3):
        ang = rng.uniform(-20, 20, size=plan.n_angles)
        psi = haar_states(rng, plan.n_in, 1)[0]
        a, oa, pa = exec_plan_dm(plan, ang, psi, noise_p=p)
        b, ob, pb = exec_plan_dm_factored(plan, ang, psi, noise_p=p)
        assert np.abs(a - b).max() < 1e-12
        assert oa == ob and np.allclose(pa, pb, atol=1e-12)


def test_factored_recurrence_outcome_one_steps():
    """prob0 below the 1e-4 threshold: the input qubit in |0> measured in
    the XZ plane near -pi/2 (projector near |1><1|) takes outcome 1."""
    circ = C.linear_cluster(6)
    circ[0] = C.Ment("XZ")
    plan = compile_plan(circ, "dm")
    assert plan.window >= 2
    rng = np.random.default_rng(4)
    seen = set()
    for d in (0.0, 1e-3, 0.019, 0.021, 0.5):
        ang = rng.uniform(0, 2 * np.pi, size=plan.n_angles)
        ang[0] = -np.pi / 2 + d
        psi = np.array([1.0, 0.0], complex)
        a, oa, _ = exec_plan_dm(plan, ang, psi)
        b, ob, _ = exec_plan_dm_factored(plan, ang, psi)
        assert oa == ob and np.abs(a - b).max() < 1e-12
        seen.add(ob[0])
    assert seen == {0, 1}
