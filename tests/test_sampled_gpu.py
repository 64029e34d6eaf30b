"""Sampled outcomes with flow byproduct corrections (force0=False)."""
import numpy as np
import pytest
import torch

from helpers import haar_states
from mentpy_gb300 import circuit as C
from mentpy_gb300.sweep import StatevectorSweep
from oracle import fullcircuit
from oracle import sweep as oracle_sweep

pytestmark = pytest.mark.gpu


def _infid(a, b):
    return 1.0 - abs(np.vdot(a / np.linalg.norm(a), b / np.linalg.norm(b))) ** 2


CIRCS = {"lin7": lambda: C.linear_cluster(7), "mw3x3": lambda: C.many_wires([3, 3, 3]),
         "grid2x4": lambda: C.grid_cluster(2, 4), "grid3x3": lambda: C.grid_cluster(3, 3)}


@pytest.mark.parametrize("name", sorted(CIRCS))
def test_sampled_matches_pennylane_semantics(name):
    """For the outcomes the kernel drew, the PennyLane circuit (restated in
    numpy: measure, then X on flow(i) and Z on later neighbours of flow(i))
    gives the same output state; with a causal flow that state is also the
    force0 state (the corrections make the pattern deterministic)."""
    circ = CIRCS[name]()
    rng = np.random.default_rng(51)
    sw = StatevectorSweep(circ)
    B = 24
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    inp = haar_states(rng, sw.n_in, B)
    st, outc, status = sw.forward_sampled(ang, inp, seed=2024)
    forced, _, _ = sw.forward(ang, inp)
    torch.cuda.synchronize()
    assert int((status != 0).sum()) == 0
    st, outc, forced = st.cpu().numpy(), outc.cpu().numpy(), forced.cpu().numpy()
    assert outc.any() and not outc.all()  # outcomes really drawn
    for r in range(B):
        oc = {node: int(o) for node, o in zip(sw.plan.schedule_measure, outc[r])}
        ref = fullcircuit.run_full_sampled_sv(circ, ang[r], inp[r], oc, sw.plan.out_nodes)
        assert _infid(st[r], ref) < 1e-5
        assert _infid(st[r], forced[r]) < 1e-5


def test_sampled_outcomes_are_reproducible_and_unbiased():
    circ = C.many_wires([5, 5])
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(53)
    B = 4096
    ang = np.tile(rng.uniform(0, 2 * np.pi, size=sw.n_angles), (B, 1))
    _, o1, _ = sw.forward_sampled(ang, None, seed=11)
    _, o2, _ = sw.forward_sampled(ang, None, seed=11)
    _, o3, _ = sw.forward_sampled(ang, None, seed=12)
    torch.cuda.synchronize()
    assert torch.equal(o1, o2) and not torch.equal(o1, o3)
    # measurements on a cluster with causal flow give 0 or 1 with probability 1/2
    frac = o1.float().mean(dim=0).cpu().numpy()
    assert np.all(np.abs(frac - 0.5) < 5 * np.sqrt(0.25 / B))


def _check_against_oracle(circ, sw, ang, inp, st, outc, runs, tol):
    for r in runs:
        oc = {node: int(o) for node, o in zip(sw.plan.schedule_measure, outc[r])}
        ref = oracle_sweep.run_sv_sampled(circ, ang[r], None if inp is None else inp[r], oc)
        assert _infid(st[r], ref) < tol, (r, _infid(st[r], ref))


@pytest.mark.parametrize("length", [150, 1001])
def test_sampled_long_sweeps(length):
    """298 and 2000 steps (the frame is a shared-memory bitset over all steps):
    against the windowed oracle with the drawn outcomes, and against the
    force0 sweep (causal-flow determinism)."""
    circ = C.many_wires([length, length])
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(54)
    B = 64
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    inp = haar_states(rng, sw.n_in, B)
    st, outc, status = sw.forward_sampled(ang, inp, seed=77)
    forced, _, _ = sw.forward(ang, inp)
    torch.cuda.synchronize()
    assert int((status != 0).sum()) == 0
    st, outc, forced = st.cpu().numpy(), outc.cpu().numpy(), forced.cpu().numpy()
    assert outc.shape == (B, sw.plan.n_steps) and outc.any() and not outc.all()
    _check_against_oracle(circ, sw, ang, inp, st, outc, range(0, B, 16), 1e-5)
    for r in range(B):
        assert _infid(st[r], forced[r]) < 1e-5


@pytest.mark.parametrize("wires,B", [(11, 24), (13, 24), (15, 200), (15, 60), (15, 24)])
def test_sampled_wide_windows(wires, B):
    """Windows 12, 14 (a block per run, the window in shared memory) and 16
    (the window in the workspace): 200 runs take a block per run slot, at
    most one slot per SM, so blocks loop over runs; 60 and 24 runs are
    smaller than the GPU and share each run among a cluster of 2 or 4
    blocks."""
    circ = C.many_wires([3] * wires)
    sw = StatevectorSweep(circ)
    assert sw.plan.window == wires + 1
    rng = np.random.default_rng(55 + wires)
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    inp = haar_states(rng, sw.n_in, B)
    st, outc, status = sw.forward_sampled(ang, inp, seed=78)
    forced, fstatus, _ = sw.forward(ang, inp)
    torch.cuda.synchronize()
    assert int((status != 0).sum()) == 0 and int((fstatus != 0).sum()) == 0
    st, outc, forced = st.cpu().numpy(), outc.cpu().numpy(), forced.cpu().numpy()
    assert outc.any() and not outc.all()
    _check_against_oracle(circ, sw, ang, inp, st, outc, [0, 1, B // 2, B - 1], 1e-5)
    for r in range(B):
        assert _infid(st[r], forced[r]) < 1e-5


def test_sampled_grid16x10_window17():
    """The streamed workload's circuit (w = 17, 144 steps): the window in the
    workspace, input placement and output gather from the plan's bit tables
    (no index map at this window)."""
    circ = C.grid_cluster(16, 10)
    sw = StatevectorSweep(circ)
    assert sw.plan.window == 17 and sw.plan.n_steps == 144
    rng = np.random.default_rng(57)
    B = 8
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    st, outc, status = sw.forward_sampled(ang, None, seed=79)
    st2, outc2, _ = sw.forward_sampled(ang, None, seed=79)
    forced, fstatus, _ = sw.forward(ang, None)
    torch.cuda.synchronize()
    assert int((status != 0).sum()) == 0 and int((fstatus != 0).sum()) == 0
    # 8 runs: a cluster of four blocks per run; the same draws and bits again
    assert torch.equal(outc, outc2) and torch.equal(st, st2)
    st, outc, forced = st.cpu().numpy(), outc.cpu().numpy(), forced.cpu().numpy()
    assert outc.any() and not outc.all()
    _check_against_oracle(circ, sw, ang, None, st, outc, [0, B - 1], 1e-5)
    for r in range(B):
        assert _infid(st[r], forced[r]) < 1e-5
