"""Named workload cases for profiling: run one kernel family a few times on
synthetic inputs (a helper of bench.py; the ncu summaries under profiles/
name the case they captured).

    python bench_cases.py <case> [--reps N]

Cases (seeded synthetic inputs with the shapes of the configuration):
  sv_mw4x8     statevector sweep, many_wires([8]*4), 4096 runs (--variant: lanes per run)
  adjoint_mw6x12 fused fidelity adjoint, many_wires([12]*6), 128 vectors x 256 inputs
  wide_grid16x10 streamed statevector, grid_cluster(16, 10), w=17, 64 runs
  adjoint_wide_grid16x10 generic adjoint of grid_cluster(16, 10), w=17, 16 runs
  dm_mw6x12    density matrix, many_wires([12]*6) (w=7), 512 runs, noise 0.01

Used for profiling (each case exits 0 when its kernels report no failed run).
"""
from __future__ import annotations

import argparse
import sys

import os

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from mentpy_gb300 import circuit as C  # noqa: E402


def _haar(rng, n, count):
    d = 2**n
    z = (rng.standard_normal((count, d, d)) + 1j * rng.standard_normal((count, d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    diag = np.diagonal(r, axis1=1, axis2=2)
    return np.ascontiguousarray((q * (diag / np.abs(diag))[:, None, :])[:, :, 0])


def case_sv_mw4x8(reps, variant=-1):
    from mentpy_gb300.sweep import StatevectorSweep

    rng = np.random.default_rng(1)
    circ = C.many_wires([8] * 4)
    sw = StatevectorSweep(circ)
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(4096, sw.n_angles)), device="cuda")
    inp = torch.as_tensor(_haar(rng, 4, 4096), dtype=torch.complex64, device="cuda")
    for _ in range(reps):
        _, st, _ = sw.forward(ang, inp, variant=variant)
    return int((st != 0).sum())


def case_sv_latency(reps):
    """One warp: 32 runs of many_wires([8]*4), one lane per run (variant 0)."""
    from mentpy_gb300.sweep import StatevectorSweep

    rng = np.random.default_rng(5)
    sw = StatevectorSweep(C.many_wires([8] * 4))
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(32, sw.n_angles)), device="cuda")
    inp = torch.as_tensor(_haar(rng, 4, 32), dtype=torch.complex64, device="cuda")
    for _ in range(reps):
        _, st, _ = sw.forward(ang, inp, variant=0)
    return int((st != 0).sum())


def case_adjoint_mw6x12(reps):
    from mentpy_gb300.sweep import StatevectorSweep

    rng = np.random.default_rng(2)
    sw = StatevectorSweep(C.many_wires([12] * 6))
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(128, sw.n_angles)), device="cuda")
    inp = torch.as_tensor(_haar(rng, 6, 256), dtype=torch.complex64, device="cuda")
    tg = torch.as_tensor(_haar(rng, 6, 256), dtype=torch.complex64, device="cuda")
    st = torch.zeros(128 * 256, dtype=torch.int32, device="cuda")
    for _ in range(reps):
        sw.fidelity_grad(ang, inp, tg, status=st)
    return int((st != 0).sum())


def case_wide_grid16x10(reps):
    from mentpy_gb300.sweep import StatevectorSweep

    rng = np.random.default_rng(3)
    sw = StatevectorSweep(C.grid_cluster(16, 10))
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(64, sw.n_angles)), device="cuda")
    for _ in range(reps):
        _, st, _ = sw.forward(ang, None)
    return int((st != 0).sum())


def case_dm_mw6x12(reps):
    from mentpy_gb300.dm import DensityMatrixSweep

    rng = np.random.default_rng(4)
    sw = DensityMatrixSweep(C.many_wires([12] * 6))
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(512, sw.n_angles)), device="cuda")
    inp = torch.as_tensor(_haar(rng, 6, 512), dtype=torch.complex64, device="cuda")
    for _ in range(reps):
        _, _, st, _ = sw.forward(ang, inp, noise=0.01)
    return int((st != 0).sum())


def case_adjoint_wide_grid16x10(reps):
    """Generic adjoint of grid_cluster(16, 10) (w = 17), 16 runs (a cluster of four blocks per run)."""
    from mentpy_gb300.sweep import StatevectorSweep

    rng = np.random.default_rng(6)
    sw = StatevectorSweep(C.grid_cluster(16, 10))
    B = 16
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles)), device="cuda")
    g = rng.standard_normal((B, 2**sw.n_out)) + 1j * rng.standard_normal((B, 2**sw.n_out))
    gout = torch.tensor(g.astype(np.complex64), device="cuda")
    st = torch.empty(B, dtype=torch.int32, device="cuda")
    for _ in range(reps):
        sw.adjoint(ang, None, gout, status=st)
    return int((st != 0).sum())


CASES = {"sv_mw4x8": case_sv_mw4x8, "sv_latency": case_sv_latency, "adjoint_mw6x12": case_adjoint_mw6x12,
         "wide_grid16x10": case_wide_grid16x10, "adjoint_wide_grid16x10": case_adjoint_wide_grid16x10,
         "dm_mw6x12": case_dm_mw6x12}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--variant", type=int, default=None,
                    help="statevector cases: log2 lanes per run of the register kernel")
    a = ap.parse_args(argv)
    kw = {} if a.variant is None else {"variant": a.variant}
    bad = CASES[a.case](a.reps, **kw)
    torch.cuda.synchronize()
    print(f"{a.case}: {a.reps} reps, failed runs {bad}")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
