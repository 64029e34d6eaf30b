"""Long sweeps: thousands of measurements against the complex128 oracle.
Renormalisation compounds over many steps (np_simulator_sv.py:351-353,
state_ops.py:73); the kernels keep complex64 amplitudes and accumulate every
norm in float pairs (about 48 significand bits), so the output stays within
the complex64 bounds and the log-probability of the all-zero branch stays
within a few complex64 roundings per step."""
import numpy as np
import pytest
import torch

from helpers import haar_states
from mentpy_gb300 import circuit as C
from mentpy_gb300.sweep import StatevectorSweep
from oracle import sweep as oracle

pytestmark = pytest.mark.gpu

TOL_INFID_C64 = 1e-5
TOL_AMP_C64 = 2e-5

LONG = {"lin2001": lambda: C.linear_cluster(2001), "mw400x4": lambda: C.many_wires([400] * 4)}


def _infid(a, b):
    a = np.asarray(a, dtype=np.complex128)
    a = a / np.linalg.norm(a, axis=-1, keepdims=True)
    b = b / np.linalg.norm(b, axis=-1, keepdims=True)
    return 1.0 - np.abs(np.sum(a.conj() * b, axis=-1)) ** 2


def _logprob_rel_tol_c64(n_steps):
    # complex64 amplitudes: each step's probability carries a relative error
    # of a few float ulps (6e-8) of accumulated amplitude rounding, which adds
    # up like a random walk over the steps; |logprob| grows like n_steps ln 2
    return 10 * 6e-8 * np.sqrt(n_steps) / (n_steps * np.log(2) * 0.5)


@pytest.mark.parametrize("name", sorted(LONG))
def test_long_sweep_complex64(name):
    circ = LONG[name]()
    sw = StatevectorSweep(circ)
    M = sw.plan.n_steps
    assert M >= 1500
    rng = np.random.default_rng(111)
    B = 64
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    out, st, lp = sw.forward(ang, psi, logprob=True)
    assert (st.cpu().numpy() == 0).all()
    ref, probs = oracle.run_sv_batch(circ, ang, psi)
    out, lp = out.cpu().numpy(), lp.cpu().numpy()
    assert _infid(out, ref).max() < TOL_INFID_C64
    assert np.abs(out - ref).max() < TOL_AMP_C64
    ref_lp = np.sum(np.log(probs), axis=1)
    rel = np.abs(lp - ref_lp) / np.abs(ref_lp)
    assert rel.max() < _logprob_rel_tol_c64(M), (rel.max(), _logprob_rel_tol_c64(M))


@pytest.mark.parametrize("name", sorted(LONG))
def test_long_sweep_fp64_check_mode(name):
    circ = LONG[name]()
    sw = StatevectorSweep(circ, dtype=torch.complex128)
    rng = np.random.default_rng(112)
    B = 16
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    out, st, lp = sw.forward(ang, psi, logprob=True)
    assert (st.cpu().numpy() == 0).all()
    ref, probs = oracle.run_sv_batch(circ, ang, psi)
    out, lp = out.cpu().numpy(), lp.cpu().numpy()
    assert _infid(out, ref).max() < 1e-12
    assert np.abs(out - ref).max() < 1e-10
    ref_lp = np.sum(np.log(probs), axis=1)
    assert (np.abs(lp - ref_lp) / np.abs(ref_lp)).max() < 1e-12
