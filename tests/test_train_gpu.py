"""Device training loop (fused fidelity adjoint + Adam) against host loops."""
import numpy as np
import pytest
import torch

from helpers import haar_states
from mentpy_gb300 import _native
from mentpy_gb300 import circuit as C
from mentpy_gb300.sweep import StatevectorSweep, _ptr, _stream_ptr
from mentpy_gb300.train import FidelityTrainer
from oracle.train import adam_step

pytestmark = pytest.mark.gpu


def test_adam_kernel_matches_reference_step():
    rng = np.random.default_rng(0)
    n = 5000
    x = rng.standard_normal(n)
    m = np.zeros(n)
    v = np.zeros(n)
    xd, md, vd = (torch.as_tensor(a, device="cuda").clone() for a in (x, m, v))
    state = torch.zeros(3, dtype=torch.float64, device="cuda")
    L = _native.lib()
    _native.check(L.mbqc_adam_state_init(_ptr(state), 0.9, 0.999, _stream_ptr(None)))
    for i in range(7):
        g = rng.standard_normal(n) * 10.0 ** rng.uniform(-6, 1, n)
        gd = torch.as_tensor(g, device="cuda")
        _native.check(L.mbqc_adam_step(n, _ptr(xd), _ptr(gd), _ptr(md), _ptr(vd), _ptr(state), 0.05, 0.9, 0.999,
                                       1e-8, _stream_ptr(None)))
        x, m, v = adam_step(x, g, m, v, i, step_size=0.05)
    torch.cuda.synchronize()
    assert float(state[0]) == 7.0
    np.testing.assert_allclose(xd.cpu().numpy(), x, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(md.cpu().numpy(), m, rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(vd.cpu().numpy(), v, rtol=1e-13, atol=1e-300)


def _problem(V=6, J=8):
    rng = np.random.default_rng(4)
    sw = StatevectorSweep(C.many_wires([4, 4]))
    x0 = rng.uniform(0, 2 * np.pi, size=(V, sw.n_angles))
    inp = haar_states(rng, sw.n_in, J)
    u = np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))[0]
    tg = inp @ u.T
    return sw, x0, inp, tg


def test_graph_replay_equals_eager_iterations():
    sw, x0, inp, tg = _problem()
    a = FidelityTrainer(sw, inp, tg, x0, step_size=0.05)
    b = FidelityTrainer(sw, inp, tg, x0, step_size=0.05)
    a.run(9, graph=True)
    b.run(9, graph=False)
    torch.cuda.synchronize()
    assert torch.equal(a.angles, b.angles)
    assert torch.equal(a.losses, b.losses)
    a.run(3, graph=True)  # continues from iteration 9
    b.run(3, graph=False)
    torch.cuda.synchronize()
    assert torch.equal(a.angles, b.angles)
    assert a.losses.shape[0] == 12 and torch.equal(a.losses, b.losses)


def test_trainer_matches_host_loop_with_reference_adam():
    sw, x0, inp, tg = _problem()
    tr = FidelityTrainer(sw, inp, tg, x0, step_size=0.05)
    tr.run(10)
    torch.cuda.synchronize()
    x = x0.copy()
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    losses = []
    for i in range(10):
        loss, grad = sw.fidelity_grad(torch.as_tensor(x, device="cuda"), inp, tg)
        losses.append(loss.cpu().numpy())
        x, m, v = adam_step(x, grad.cpu().numpy(), m, v, i, step_size=0.05)
    # the two loops feed the complex64 kernel angles that differ in the last
    # FP64 bits (device vs numpy Adam), so agreement is to float precision
    np.testing.assert_allclose(tr.angles.cpu().numpy(), x, rtol=0, atol=1e-6)
    np.testing.assert_allclose(tr.losses.cpu().numpy(), np.array(losses), rtol=0, atol=1e-6)


def test_training_lowers_the_loss():
    sw, x0, inp, tg = _problem(V=16)
    tr = FidelityTrainer(sw, inp, tg, x0, step_size=0.05)
    tr.run(200)
    torch.cuda.synchronize()
    first, last = tr.losses[0], tr.losses[-1]
    assert int((tr.status != 0).sum()) == 0
    assert float((last < first).float().mean()) > 0.9
