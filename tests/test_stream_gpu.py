"""Wide-window (streamed) statevector sweep: against the register kernel where
both apply and against the complex128 oracle up to window 17."""
import numpy as np
import pytest
import torch

from helpers import haar_states
from mentpy_gb300 import circuit as C
from mentpy_gb300.sweep import STREAMED, StatevectorSweep
from oracle import sweep as oracle

pytestmark = pytest.mark.gpu

TOL_AMP_C64 = 2e-5


def _infid(a, b):
    return 1.0 - abs(np.vdot(a / np.linalg.norm(a), b / np.linalg.norm(b))) ** 2


@pytest.mark.parametrize("build", [lambda: C.grid_cluster(7, 4), lambda: C.grid_cluster(8, 5),
                                   lambda: C.grid_cluster(9, 4), lambda: C.many_wires([6] * 8)])
def test_streamed_equals_register_kernel(build):
    circ = build()
    sw = StatevectorSweep(circ)
    assert 8 <= sw.plan.window <= 10
    rng = np.random.default_rng(3)
    B = 37
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    a, sa, la = sw.forward(ang, psi, logprob=True)
    b, sb, lb = sw.forward(ang, psi, logprob=True, variant=STREAMED)
    assert (sa == 0).all() and (sb == 0).all()
    assert (a - b).abs().max().item() < 1e-5
    assert (la - lb).abs().max().item() < 1e-4


@pytest.mark.parametrize("rows,cols,B", [(10, 4, 6), (11, 6, 5), (12, 3, 4), (13, 4, 3), (16, 10, 64), (19, 3, 2)])
def test_wide_window_against_oracle(rows, cols, B):
    circ = C.grid_cluster(rows, cols)
    sw = StatevectorSweep(circ)
    assert sw.plan.window == rows + 1
    rng = np.random.default_rng(rows * 100 + cols)
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = None if rows >= 16 else haar_states(rng, sw.n_in, B)
    out, st, _ = sw.forward(ang, psi)
    out = out.cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    assert np.abs(np.linalg.norm(out, axis=1) - 1).max() < 1e-5
    for r in rng.choice(B, min(B, 2), replace=False):
        ref, _, _ = oracle.run_sv(circ, ang[r], None if psi is None else psi[r], output_form="sv")
        assert _infid(out[r], ref) < 1e-5
        assert np.abs(out[r] - ref).max() < TOL_AMP_C64
    out2, _, _ = sw.forward(ang, psi)
    assert np.array_equal(out, out2.cpu().numpy())


def test_streamed_logprob_multichunk_against_oracle():
    """More outputs than one epilogue chunk (2^10): the all-zero-branch
    log-probability sums the run's chunk partials, against the oracle's
    per-step probabilities."""
    circ = C.grid_cluster(12, 3)
    sw = StatevectorSweep(circ)
    assert sw.plan.window == 13 and sw.n_out == 12
    rng = np.random.default_rng(41)
    B = 3
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    out, st, lp = sw.forward(ang, psi, logprob=True)
    assert (st.cpu().numpy() == 0).all()
    lp = lp.cpu().numpy()
    for r in range(B):
        ref, _, probs = oracle.run_sv(circ, ang[r], psi[r], output_form="sv")
        assert abs(lp[r] - np.sum(np.log(probs))) < 1e-4
        assert _infid(out[r].cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("rows,cols", [(10, 4), (13, 4), (16, 10)])
def test_tma_staging_gives_the_same_bits(rows, cols):
    """Mixed passes staged by TMA bulk copies (MBQC_F_STREAM_TMA) and by
    16-byte asynchronous copies compute the same arithmetic on the same data."""
    circ = C.grid_cluster(rows, cols)
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(rows + cols)
    B = 8 if rows < 16 else 4
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = None if rows >= 16 else haar_states(rng, sw.n_in, B)
    a, sa, la = sw.forward(ang, psi, logprob=True)
    b, sb, lb = sw.forward(ang, psi, logprob=True, stream_tma=True)
    assert (sa == 0).all() and (sb == 0).all()
    assert torch.equal(a, b) and torch.equal(la, lb)
