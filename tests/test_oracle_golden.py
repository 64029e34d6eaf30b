"""Pin the oracle: the complex128 restatement and the dense port reproduce the
reference's outputs (stored fixtures) on every golden case."""
import numpy as np
import pytest

from helpers import circuit_from_spec, golden_names, load_golden
from oracle import sweep
from oracle.dense import DenseSV


def _inputs(data, r):
    return data["inputs"][r] if "inputs" in data else None


@pytest.mark.parametrize("name", golden_names())
def test_sweep_sv_matches_reference(name):
    spec, data = load_golden(name)
    if "sv_state" not in data:
        pytest.skip("no numpy-sv output for this case")
    circ = circuit_from_spec(spec)
    kw = spec["sim_kwargs"]
    for r in range(len(data["angles"])):
        st, outc, _ = sweep.run_sv(circ, data["angles"][r], _inputs(data, r), output_form="sv", **kw)
        ref = data["sv_state"][r]
        # amplitudes, including the reference's global phase
        assert np.allclose(st, ref, atol=1e-10), name
        assert list(outc.keys()) == spec["sv_outcome_nodes"]
        assert list(outc.values()) == list(data["sv_outcomes"][r])


@pytest.mark.parametrize("name", golden_names())
def test_sweep_dm_matches_reference(name):
    spec, data = load_golden(name)
    if "dm_rho" not in data:
        pytest.skip("no numpy-dm output for this case")
    circ = circuit_from_spec(spec)
    kw = spec["sim_kwargs"]
    mode = spec.get("dm_mode", "sample")
    for r in range(len(data["angles"])):
        rho, outc, _ = sweep.run_dm(circ, data["angles"][r], _inputs(data, r), mode=mode, **kw)
        assert np.allclose(rho, data["dm_rho"][r], atol=1e-10), name
        assert list(outc.keys()) == spec["dm_outcome_nodes"]
        if "dm_zexp_outcomes" in data:  # expectation mode: Z entries are prob1 / (prob0 + prob1)
            assert np.allclose(list(outc.values()), data["dm_zexp_outcomes"][r], atol=1e-10)
        else:
            assert list(outc.values()) == list(data["dm_outcomes"][r])


@pytest.mark.parametrize("name", ["lin9", "mw4x8", "grid3x5", "lin7_fixed", "rand_muta21_1_w5"])
def test_dense_port_matches_reference(name):
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    sim = DenseSV(circ, **spec["sim_kwargs"])
    for r in range(len(data["angles"])):
        rho = sim.run(data["angles"][r], _inputs(data, r))
        ref = np.outer(data["sv_state"][r], data["sv_state"][r].conj())
        assert np.allclose(rho, ref, atol=1e-10)


def test_sv_dm_cross_check():
    """numpy-sv and numpy-dm agree (the reference's cross-backend check)."""
    for name in ["grid3x5", "mw4x8", "rand_grid2x5_w5_xx"]:
        spec, data = load_golden(name)
        for r in range(len(data["angles"])):
            sv = data["sv_state"][r]
            assert np.allclose(np.outer(sv, sv.conj()), data["dm_rho"][r], atol=1e-10)


def test_teleportation_identity():
    for n in (3, 5, 7, 9):
        spec, data = load_golden(f"teleport_lin{n}")
        for r in range(3):
            st = data["inputs"][r]
            assert np.allclose(data["dm_rho"][r], np.outer(st, st.conj()), atol=1e-3)


@pytest.mark.parametrize("name", golden_names())
def test_batched_oracle_matches_reference(name):
    """The vectorised restatement (whole benchmark batches are checked with
    it) reproduces the same fixtures as the per-run one."""
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    kw = spec["sim_kwargs"]
    inputs = data.get("inputs")
    if "sv_state" in data:
        st, probs = sweep.run_sv_batch(circ, data["angles"], inputs, **kw)
        assert np.allclose(st, data["sv_state"], atol=1e-10), name
    if "dm_rho" in data and "dm_zexp_outcomes" not in data:
        if any(m[1] == "Z" for m in spec["measurements"]):
            return
        rho, outc, _ = sweep.run_dm_batch(circ, data["angles"], inputs, **kw)
        assert np.allclose(rho, data["dm_rho"], atol=1e-10), name
        # outcome columns in the reference's dict order (measured nodes first)
        n_meas = outc.shape[1]
        assert np.array_equal(outc, data["dm_outcomes"][:, :n_meas]), name
