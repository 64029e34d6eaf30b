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
    # gradients and drawn outcomes take XY, X and Y steps only
    sw = StatevectorSweep(circ, extended_planes=True)
    with pytest.raises(_native.MbqcError):
        sw.adjoint(data["angles"][:1], data["inputs"][:1], np.ones((1, 2), np.complex64))
