"""Noise model pinning (CPU): the windowed density-matrix sweep with the
per-qubit depolarising placement equals the whole-graph simulation with
PennyLane's placement; without noise both equal the reference fixtures."""
import numpy as np
import pytest

from helpers import circuit_from_spec, exec_plan_dm, haar_states, load_golden
from mentpy_gb300 import circuit as C
from mentpy_gb300.plan import compile_plan
from oracle import fullcircuit, sweep


@pytest.mark.parametrize("build", [lambda: C.linear_cluster(5), lambda: C.many_wires([3, 3]),
                                   lambda: C.grid_cluster(2, 3), lambda: C.grid_cluster(2, 4)])
@pytest.mark.parametrize("p", [0.0, 0.01, 0.2])
def test_windowed_noise_equals_full_circuit(build, p):
    circ = build()
    rng = np.random.default_rng(4)
    ang = rng.uniform(0, 2 * np.pi, len(circ.trainable_nodes))
    psi = haar_states(rng, len(circ.input_nodes), 1)[0]
    win, _, _ = sweep.run_dm(circ, ang, psi, noise_p=p)
    full = fullcircuit.run_full_dm(circ, ang, psi, noise_p=p)
    assert np.allclose(win, full, atol=1e-10)
    plan = compile_plan(circ, "dm")
    rho, _, _ = exec_plan_dm(plan, ang, psi, noise_p=p)
    assert np.allclose(rho, full, atol=1e-10)


@pytest.mark.parametrize("name", ["lin9_haar", "rand_grid2x4_w5", "teleport_lin7"])
def test_full_circuit_matches_reference_without_noise(name):
    # whole-graph simulation is 4^N: small graphs only
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    for r in range(2):
        inp = data["inputs"][r] if "inputs" in data else None
        full = fullcircuit.run_full_dm(circ, data["angles"][r], inp)
        assert np.allclose(full, data["dm_rho"][r], atol=1e-10)
