"""The benchmark batches themselves against the complex128 oracle, every run:
many_wires([8]*4) x 4096 (angle vector, Haar input) pairs, and the uneven
batch of 2048 noisy density-matrix circuits with bit-exact outcome
bookkeeping (1 iff prob0 < 1e-4, np_simulator_dm.py:335-338)."""
import numpy as np
import pytest
import torch

from helpers import haar_states
from mentpy_gb300 import circuit as C
from mentpy_gb300.dm import UnevenDensityMatrixBatch
from mentpy_gb300.native_plan import GraphBatch
from mentpy_gb300.sweep import StatevectorSweep
from oracle import sweep as oracle

pytestmark = pytest.mark.gpu

TOL_INFID_C64 = 1e-5
TOL_AMP_C64 = 2e-5
TOL_RHO_C64 = 2e-5


def _infid(a, b):
    a = np.asarray(a, dtype=np.complex128)
    a = a / np.linalg.norm(a, axis=-1, keepdims=True)
    b = b / np.linalg.norm(b, axis=-1, keepdims=True)
    return 1.0 - np.abs(np.sum(a.conj() * b, axis=-1)) ** 2


@pytest.mark.parametrize("lo,hi", [(0.0, 2 * np.pi), (-1e4, 1e4)])
def test_full_statevector_batch_against_oracle(lo, hi):
    circ = C.many_wires([8] * 4)
    rng = np.random.default_rng(121)
    B = 4096
    ang = rng.uniform(lo, hi, size=(B, len(circ.trainable_nodes)))
    psi = haar_states(rng, 4, B)
    sw = StatevectorSweep(circ)
    out, st, lp = sw.forward(ang, psi, logprob=True)
    assert (st.cpu().numpy() == 0).all()
    ref, probs = oracle.run_sv_batch(circ, ang, psi)
    out, lp = out.cpu().numpy(), lp.cpu().numpy()
    assert _infid(out, ref).max() < TOL_INFID_C64
    assert np.abs(out - ref).max() < TOL_AMP_C64  # the reference's global phase included
    assert np.abs(lp - np.sum(np.log(probs), axis=1)).max() < 1e-5


def test_full_uneven_density_matrix_batch_against_oracle():
    rng = np.random.default_rng(122)
    n = 2048
    shapes = [(int(rng.integers(2, 7)), int(rng.integers(4, 13))) for _ in range(n)]
    ub = UnevenDensityMatrixBatch.from_graph_batch(GraphBatch.many_wires(shapes))
    buf = ub.allocate()
    angs, psis = [], []
    for c, p in enumerate(ub.plans):
        a = rng.uniform(0, 2 * np.pi, p.n_angles)
        v = haar_states(rng, p.n_in, 1)[0]
        angs.append(a)
        psis.append(v)
        buf["angles"][c, : p.n_angles] = torch.as_tensor(a)
        buf["inputs"][c, : 2**p.n_in] = torch.as_tensor(v, dtype=torch.complex64)
    ub.capture(buf, noise=0.01)
    ub.run(buf, noise=0.01)
    torch.cuda.synchronize()
    assert int((buf["status"] != 0).sum()) == 0
    rho_all = buf["rho"].cpu().numpy()
    outc_all = buf["outcomes"].cpu().numpy()
    # the oracle, one vectorised call per circuit shape
    by_shape = {}
    for c, s in enumerate(shapes):
        by_shape.setdefault(s, []).append(c)
    worst = 0.0
    for (W, D), idx in by_shape.items():
        circ = C.many_wires([D] * W)
        ref, ref_out, _ = oracle.run_dm_batch(circ, np.stack([angs[c] for c in idx]),
                                              np.stack([psis[c] for c in idx]), noise_p=0.01)
        d = ref.shape[1]
        for j, c in enumerate(idx):
            M = ub.plans[c].n_steps
            got = rho_all[c, : d * d].reshape(d, d)
            worst = max(worst, float(np.abs(got - ref[j]).max()))
            assert np.array_equal(outc_all[c, :M], ref_out[j]), (W, D, c)
    assert worst < TOL_RHO_C64, worst


def test_uneven_density_matrix_outcome_threshold_bit_exact():
    """Circuits whose steps sit around the outcome threshold: window 1 with
    an explicit schedule leaves the second measured qubit a bare |+>, so
    prob0 = cos^2(theta/2) and theta near pi puts it near 1e-4.  The batch
    reproduces the oracle's outcome bits on both sides of the threshold."""
    from mentpy_gb300.dm import DensityMatrixSweep

    circ = C.linear_cluster(4)
    sw = DensityMatrixSweep(circ, window_size=1, schedule=[0, 1, 2, 3])
    rng = np.random.default_rng(123)
    B = 2048
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    # 2 arccos(sqrt(p)) for prob0 p spread over [0.5e-4, 2e-4] (excluding a band of
    # float rounding around the threshold, where complex64 cannot decide)
    p = np.exp(rng.uniform(np.log(0.5e-4), np.log(2e-4), size=B))
    p = p[np.abs(p - 1e-4) > 2e-8 * 10][: B // 2]
    ang[: len(p), 1] = 2 * np.arccos(np.sqrt(p))
    rho, outc, st, _ = sw.forward(ang, None)
    ref, ref_out, _ = oracle.run_dm_batch(circ, ang, None, window_size=1, schedule=[0, 1, 2, 3])
    assert (st.cpu().numpy() == 0).all()
    outc = outc.cpu().numpy()
    assert outc[:, 1].any() and not outc[:, 1].all()
    assert np.array_equal(outc, ref_out)
    assert np.abs(rho.cpu().numpy() - ref).max() < TOL_RHO_C64
