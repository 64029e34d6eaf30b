"""The window-plan compiler: executing the plan with the kernels' in-place
conventions (tests/helpers.exec_plan_*) reproduces the reference fixtures."""
import json
import os

import numpy as np
import pytest

from helpers import (GOLDEN, circuit_from_spec, exec_plan_dm, exec_plan_sv,
                     golden_names, load_golden)
from mentpy_gb300 import circuit as C
from mentpy_gb300.plan import DEAD, compile_plan


def _inputs(spec, data, r):
    if "inputs" in data:
        return data["inputs"][r]
    n = len(spec["input_nodes"])
    return np.ones(2**n) / np.sqrt(2**n)


@pytest.mark.parametrize("name", golden_names())
def test_plan_sv(name):
    spec, data = load_golden(name)
    if "sv_state" not in data:
        pytest.skip("no numpy-sv output")
    plan = compile_plan(circuit_from_spec(spec), "sv", **spec["sim_kwargs"])
    assert plan.outcome_nodes() == spec["sv_outcome_nodes"]
    for r in range(len(data["angles"])):
        out = exec_plan_sv(plan, data["angles"][r], _inputs(spec, data, r))
        assert np.allclose(out, data["sv_state"][r], atol=1e-10), name


@pytest.mark.parametrize("name", golden_names())
def test_plan_dm(name):
    spec, data = load_golden(name)
    if "dm_rho" not in data:
        pytest.skip("no numpy-dm output")
    if spec.get("dm_mode") == "expectation":
        pytest.skip("Z-basis expectation mode: checked by the oracle and GPU tests")
    plan = compile_plan(circuit_from_spec(spec), "dm", **spec["sim_kwargs"])
    assert plan.outcome_nodes() == spec["dm_outcome_nodes"]
    for r in range(len(data["angles"])):
        rho, outc, _ = exec_plan_dm(plan, data["angles"][r], _inputs(spec, data, r))
        assert np.allclose(rho, data["dm_rho"][r], atol=1e-10), name
        assert outc == list(data["dm_outcomes"][r])


def test_plan_errors_match_reference():
    with open(os.path.join(GOLDEN, "errors.json")) as f:
        ref = json.load(f)
    c = C.linear_cluster(5)
    with pytest.raises(NotImplementedError, match=ref["force0_false"][1]):
        compile_plan(c, "sv", force0=False)
    with pytest.raises(ValueError, match=ref["window_too_big"][1]):
        compile_plan(c, "sv", window_size=9)
    spec, _ = load_golden("dm_planes_lin5")
    with pytest.raises(ValueError, match=spec["errors"]["sv"][1].split(",")[0]):
        compile_plan(circuit_from_spec(spec), "sv")


def test_plan_shapes_grid16x10():
    g = C.grid_cluster(16, 10)
    plan = compile_plan(g, "sv")
    assert plan.window == 17 and plan.n_steps == 144 and plan.n_angles == 144
    dead = sum(1 for m in plan.step_mask if m & DEAD)
    assert dead == plan.window - plan.n_out
    assert sorted(plan.out_bits.tolist()) == sorted(set(plan.out_bits.tolist()))
