"""The allocation-free adjoint entry point (mbqc_sv_adjoint_noalloc).

Callers that cannot allocate device memory — plugins inside a framework that
owns the GPU memory pool, fixed-footprint services, loops that cannot afford
cudaFree's device-wide synchronisation — use this variant: its checkpoint
scratch is a fixed array inside the library.  These tests call it through the
C ABI and check it against mbqc_sv_adjoint (which takes a caller workspace) on
two calls in a row, so that a second call on the reused array is covered too.
The file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from helpers import haar_states
from mentpy_gb300 import _native
from mentpy_gb300 import circuit as C
from mentpy_gb300.plan import DEAD, WindowPlan, compile_plan
from mentpy_gb300.sweep import StatevectorSweep

pytestmark = pytest.mark.gpu

TOL = 1e-9  # same kernel and arithmetic as the workspace variant


def _p(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("build,batch", [(lambda: C.many_wires([12] * 6), 3000),
                                         (lambda: C.many_wires([8] * 4), 513),
                                         (lambda: C.grid_cluster(3, 5), 40)])
def test_noalloc_matches_workspace_adjoint_twice(build, batch):
    circ = build()
    sw = StatevectorSweep(circ)
    rng = np.random.default_rng(99)
    A, d_in, d_out = sw.n_angles, 2 ** sw.n_in, 2 ** sw.n_out
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(batch, A)), device="cuda")
    inp = torch.as_tensor(haar_states(rng, sw.n_in, batch), dtype=torch.complex64, device="cuda")
    g = torch.as_tensor(rng.standard_normal((batch, d_out)) + 1j * rng.standard_normal((batch, d_out)),
                        dtype=torch.complex64, device="cuda")
    ref = sw.adjoint(ang, inp, g)  # mbqc_sv_adjoint with a workspace
    lib = _native.lib()
    for _ in range(2):
        grad = torch.full((batch, A), float("nan"), dtype=torch.float64, device="cuda")
        status = torch.full((batch,), -1, dtype=torch.int32, device="cuda")
        rc = lib.mbqc_sv_adjoint_noalloc(sw.dplan.handle, batch, _p(ang), A, _p(inp), d_in, _p(g), _p(grad),
                                         _p(status), _stream())
        _native.check(rc)
        torch.cuda.synchronize()
        assert (status == 0).all()
        assert (grad - ref).abs().max().item() < TOL


def test_noalloc_rejects_a_circuit_beyond_shared_memory():
    # window 8, 70000 steps: the per-run step tables exceed shared memory (the
    # binding limit: a circuit that fits it never exceeds the fixed scratch);
    # the call must fail cleanly with an explanation and leave the outputs
    # untouched
    w, M = 8, 70000
    mask = np.zeros(M, dtype=np.uint32)
    mask[-(w - 1):] = DEAD
    plan = WindowPlan(kind="sv", window=w, n_nodes=M + 1, schedule=list(range(M + 1)),
                      schedule_measure=list(range(M)), n_in=1, n_out=1, n_angles=0, trainable_nodes=[],
                      in_bits=np.array([0], np.int32), init_cz=np.zeros(w, np.uint32), step_mask=mask,
                      step_angle=np.full(M, -1, np.int32), step_plane=np.zeros(M, np.int32),
                      step_fixed_angle=np.zeros(M), out_bits=np.array([M % w], np.int32), out_nodes=[M])
    dplan = _native.DevicePlan(plan)
    inp = torch.ones((1, 2), dtype=torch.complex64, device="cuda")
    g = torch.ones((1, 2), dtype=torch.complex64, device="cuda")
    grad = torch.zeros((1, 1), dtype=torch.float64, device="cuda")
    rc = _native.lib().mbqc_sv_adjoint_noalloc(dplan.handle, 1, None, 1, _p(inp), 2, _p(g), _p(grad), None,
                                               _stream())
    assert rc == -3  # MBQC_E_UNSUPPORTED
    msg = _native.lib().mbqc_last_error().decode()
    assert "adjoint_noalloc" in msg and "shared memory" in msg
    torch.cuda.synchronize()
    assert (grad == 0).all()
