"""XZ / YZ measurements in the statevector kernels (register, FP64 check
mode, streamed) against the complex128 oracle and the reference's
density-matrix fixture; the statevector front-end keeps the reference's
rejection unless asked (np_simulator_sv.py:53-59)."""
import numpy as np
import pytest
import torch

from helpers import circuit_from_spec, haar_states, load_golden
from mentpy_gb300 import _native
from mentpy_gb300 import circuit as C
from mentpy_gb300.simulators import PatternSimulator
from mentpy_gb300.sweep import STREAMED, StatevectorSweep
from oracle import sweep as oracle

pytestmark = pytest.mark.gpu

TOL_AMP_C64 = 2e-5


def _with_planes(circ, rng, frac=0.4):
    nodes = [n for n in circ.trainable_nodes]
    for n in rng.choice(nodes, max(1, int(frac * len(nodes))), replace=False):
        circ[int(n)] = C.Ment(str(rng.choice(["XZ", "YZ"])))
    return circ


@pytest.mark.parametrize("build", [lambda: C.linear_cluster(9), lambda: C.many_wires([8] * 4),
                                   lambda: C.grid_cluster(3, 5), lambda: C.many_wires([6] * 7)])
def test_register_kernel_xz_yz(build):
    rng = np.random.default_rng(81)
    circ = _with_planes(build(), rng)
    sw = StatevectorSweep(circ, extended_planes=True)
    B = 64
    ang = rng.uniform(-20, 20, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    out, st, lp = sw.forward(ang, psi, logprob=True)
    assert (st.cpu().numpy() == 0).all()
    ref, probs = oracle.run_sv_batch(circ, ang, psi)
    assert np.abs(out.cpu().numpy() - ref).max() < TOL_AMP_C64  # global phase included
    assert np.abs(lp.cpu().numpy() - np.log(probs).sum(axis=1)).max() < 1e-4
    f64 = StatevectorSweep(circ, extended_planes=True, dtype=torch.complex128)
    o64, s64, _ = f64.forward(ang, psi)
    assert (s64.cpu().numpy() == 0).all()
    assert np.abs(o64.cpu().numpy() - ref).max() < 1e-10


@pytest.mark.parametrize("rows,cols", [(8, 4), (11, 4)])
def test_streamed_kernel_xz_yz(rows, cols):
    rng = np.random.default_rng(82)
    circ = _with_planes(C.grid_cluster(rows, cols), rng, 0.3)
    sw = StatevectorSweep(circ, extended_planes=True)
    B = 3
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    out, st, _ = sw.forward(ang, psi, variant=STREAMED)
    assert (st.cpu().numpy() == 0).all()
    ref, _ = oracle.run_sv_batch(circ, ang, psi)
    assert np.abs(out.cpu().numpy() - ref).max() < TOL_AMP_C64


def test_reference_density_matrix_fixture_and_dropin():
    spec, data = load_golden("dm_planes_lin5")
    circ = circuit_from_spec(spec)
    with pytest.raises(ValueError):
        PatternSimulator(circ, backend="cuda-sv")  # the reference's rejection by default
    ps = PatternSimulator(circ, backend="cuda-sv", extended_planes=True)
    for r in range(len(data["angles"])):
        ps.reset(input_state=data["inputs"][r])
        rho = ps.run(data["angles"][r])  # output_form="dm"
        assert np.abs(rho - data["dm_rho"][r]).max() < TOL_AMP_C64
    # gradients take these planes (the block-per-run adjoint); drawn outcomes
    # (the PennyLane backend's semantics) XY, X and Y steps only
    from oracle import gradients as G

    sw = StatevectorSweep(circ, extended_planes=True)
    gout = np.ones((1, 2), np.complex64)
    grad = sw.adjoint(data["angles"][:1], data["inputs"][:1], gout).cpu().numpy()
    ref = G.linear_functional_grad(circ, data["angles"][0], data["inputs"][0], gout[0].astype(complex), h=1e-4)
    assert np.abs(grad[0] - ref).max() < 2e-4 * (1 + np.abs(ref).max())
    with pytest.raises(_native.MbqcError):
        sw.forward_sampled(data["angles"][:1], data["inputs"][:1], seed=1, circuit=circ)


@pytest.mark.parametrize("build", [lambda: C.linear_cluster(7), lambda: C.many_wires([5] * 3),
                                   lambda: C.many_wires([3] * 9)])
def test_adjoint_xz_yz(build):
    """The adjoint of plans with XZ / YZ steps (the block-per-run kernel, both
    coefficients differentiated) against complex128 central differences of
    the oracle, and the fused fidelity gradient."""
    from oracle import gradients as G

    rng = np.random.default_rng(84)
    circ = _with_planes(build(), rng)
    sw = StatevectorSweep(circ, extended_planes=True)
    B = 2
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    g = rng.standard_normal((B, 2**sw.n_out)) + 1j * rng.standard_normal((B, 2**sw.n_out))
    st = torch.empty(B, dtype=torch.int32, device="cuda")
    grad = sw.adjoint(ang, psi, g, status=st).cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    for r in range(B):
        ref = G.linear_functional_grad(circ, ang[r], psi[r], g[r], h=1e-4)
        err = np.abs(grad[r] - ref).max() / (1 + np.abs(ref).max())
        assert err < 2e-4, (r, err)
    tg = haar_states(rng, sw.n_out, 3)
    inp = haar_states(rng, sw.n_in, 3)
    loss, fgrad = sw.fidelity_grad(ang[:1], inp, tg)
    assert abs(float(loss[0]) - G.fidelity_loss(circ, ang[0], inp, tg)) < 1e-5
    ref = G.fidelity_grad(circ, ang[0], inp, tg, h=1e-4)
    assert np.abs(fgrad[0].cpu().numpy() - ref).max() < 2e-4
