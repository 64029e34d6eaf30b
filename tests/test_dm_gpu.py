"""Density-matrix kernels against the reference fixtures, the noisy oracle and
the uneven multi-circuit batch."""
import numpy as np
import pytest
import torch

from helpers import circuit_from_spec, golden_names, haar_states, load_golden
from mentpy_gb300 import circuit as C
from mentpy_gb300.dm import CudaSimulatorDM, DensityMatrixSweep, UnevenDensityMatrixBatch
from mentpy_gb300.plan import compile_plan
from mentpy_gb300.simulators import PatternSimulator
from oracle import sweep as oracle

pytestmark = pytest.mark.gpu

TOL_RHO_C64 = 2e-5  # max |rho_gpu - rho_ref| for complex64 density matrices

DM_CASES = [n for n in golden_names() if "dm_rho" in load_golden(n)[1]]


@pytest.mark.parametrize("name", DM_CASES)
def test_dm_matches_reference(name):
    spec, data = load_golden(name)
    circ = circuit_from_spec(spec)
    sw = DensityMatrixSweep(circ, **spec["sim_kwargs"])
    mode = spec.get("dm_mode", "sample")
    rho, outc, status, probs = sw.forward(data["angles"], data.get("inputs"), want_probs=True, mode=mode)
    torch.cuda.synchronize()
    assert (status.cpu().numpy() == 0).all()
    rho, outc, probs = rho.cpu().numpy(), outc.cpu().numpy(), probs.cpu().numpy()
    for r in range(len(data["angles"])):
        assert np.abs(rho[r] - data["dm_rho"][r]).max() < TOL_RHO_C64, name
        if "dm_zexp_outcomes" in data:
            # expectation mode: Z entries (marker 2) carry prob1 / (prob0 + prob1)
            ref = data["dm_zexp_outcomes"][r]
            for k in range(len(ref)):
                if outc[r][k] == 2:
                    assert abs(probs[r][k] - ref[k]) < 1e-5, name
                else:
                    assert outc[r][k] == ref[k], name
            continue
        # outcome bookkeeping is exact (1 iff prob0 < 1e-4)
        assert list(outc[r]) == list(data["dm_outcomes"][r]), name
        _, _, ref_probs = oracle.run_dm(circ, data["angles"][r], data["inputs"][r] if "inputs" in data else None,
                                        **spec["sim_kwargs"])
        assert np.allclose(probs[r], ref_probs, atol=1e-5)


@pytest.mark.parametrize("build", [lambda: C.many_wires([6] * 3), lambda: C.grid_cluster(3, 4),
                                   lambda: C.many_wires([5] * 6), lambda: C.grid_cluster(4, 3)])
@pytest.mark.parametrize("p", [0.01, 0.2])
def test_dm_noise_matches_oracle(build, p):
    circ = build()
    rng = np.random.default_rng(8)
    B = 6
    ang = rng.uniform(0, 2 * np.pi, size=(B, len(circ.trainable_nodes)))
    psi = haar_states(rng, len(circ.input_nodes), B)
    sw = DensityMatrixSweep(circ)
    rho, outc, status, _ = sw.forward(ang, psi, noise=p)
    rho = rho.cpu().numpy()
    for r in range(B):
        ref, _, _ = oracle.run_dm(circ, ang[r], psi[r], noise_p=p)
        assert np.abs(rho[r] - ref).max() < TOL_RHO_C64


def test_dm_agrees_with_sv():
    circ = C.grid_cluster(3, 4)
    rng = np.random.default_rng(2)
    ang = rng.uniform(0, 2 * np.pi, size=(16, len(circ.trainable_nodes)))
    psi = haar_states(rng, 3, 16)
    rho, _, _, _ = DensityMatrixSweep(circ).forward(ang, psi)
    from mentpy_gb300.sweep import StatevectorSweep

    sv, _, _ = StatevectorSweep(circ).forward(ang, psi)
    ref = torch.einsum("bi,bj->bij", sv, sv.conj())
    assert (rho - ref).abs().max().item() < 1e-5


def test_cuda_dm_dropin_and_nan_error():
    rng = np.random.default_rng(12)
    for n in (3, 5, 7):
        ps = PatternSimulator(C.linear_cluster(n), backend="cuda-dm")
        for st in haar_states(rng, 1, 2):
            ps.reset(input_state=st)
            out = ps([0] * (n - 1))
            assert np.allclose(out, np.outer(st, st.conj()), atol=1e-5)
            assert set(ps.outcomes.values()) == {0}
    ps = PatternSimulator(C.linear_cluster(5), backend="cuda-dm")
    with pytest.raises(ValueError, match="qstate has nan"):
        ps.run([0.1, float("nan"), 0.2, 0.3])
    ps.reset()
    with pytest.raises(ValueError, match="Number of angles"):
        ps.run([0.1])


def _random_many_wires(rng, n):
    circs = []
    for _ in range(n):
        W = int(rng.integers(2, 7))
        D = int(rng.integers(4, 13))
        circs.append(C.many_wires([D] * W))
    return circs


def test_uneven_batch_matches_oracle_and_graph_replay():
    rng = np.random.default_rng(21)
    circs = _random_many_wires(rng, 24)
    plans = [compile_plan(c, "dm") for c in circs]
    ub = UnevenDensityMatrixBatch(plans)
    buf = ub.allocate()
    angs, psis = [], []
    for c, (circ, plan) in enumerate(zip(circs, plans)):
        a = rng.uniform(0, 2 * np.pi, size=plan.n_angles)
        psi = haar_states(rng, plan.n_in, 1)[0]
        buf["angles"][c, : plan.n_angles] = torch.as_tensor(a)
        buf["inputs"][c, : 2**plan.n_in] = torch.as_tensor(psi, dtype=torch.complex64)
        angs.append(a)
        psis.append(psi)
    ub.run(buf, noise=0.01)
    torch.cuda.synchronize()
    assert (buf["status"] == 0).all()
    first = buf["rho"].clone()
    for c, circ in enumerate(circs):
        ref, outc, _ = oracle.run_dm(circ, angs[c], psis[c], noise_p=0.01)
        assert np.abs(ub.rho(buf, c).cpu().numpy() - ref).max() < TOL_RHO_C64
        M = plans[c].n_steps
        assert list(buf["outcomes"][c, :M].cpu().numpy()) == list(outc.values())
    buf["rho"].zero_()
    ub.capture(buf, noise=0.01)
    buf["rho"].zero_()
    ub.run(buf, noise=0.01)  # graph replay
    torch.cuda.synchronize()
    assert torch.equal(buf["rho"], first)


def test_uneven_batch_from_native_graph_batch_matches_python_plans():
    """Plans compiled natively from flat graph arrays drive the kernels to the
    same bits as plans from the Python compiler."""
    from mentpy_gb300.dm import UnevenDensityMatrixBatch
    from mentpy_gb300.native_plan import GraphBatch

    rng = np.random.default_rng(31)
    shapes = [(int(rng.integers(2, 7)), int(rng.integers(4, 13))) for _ in range(96)]
    py = UnevenDensityMatrixBatch([compile_plan(C.many_wires([d] * w), "dm") for w, d in shapes])
    nat = UnevenDensityMatrixBatch.from_graph_batch(GraphBatch.many_wires(shapes))
    b1, b2 = py.allocate(), nat.allocate()
    for c, p in enumerate(py.plans):
        ang = torch.as_tensor(rng.uniform(0, 2 * np.pi, p.n_angles))
        v = rng.standard_normal(2 ** p.n_in) + 1j * rng.standard_normal(2 ** p.n_in)
        inp = torch.as_tensor(v / np.linalg.norm(v), dtype=torch.complex64)
        for b in (b1, b2):
            b["angles"][c, : p.n_angles] = ang
            b["inputs"][c, : 2 ** p.n_in] = inp
    py.run(b1, noise=0.01)
    nat.run(b2, noise=0.01)
    torch.cuda.synchronize()
    assert int((b1["status"] != 0).sum()) == 0
    assert torch.equal(b1["rho"], b2["rho"])
    assert torch.equal(b1["outcomes"], b2["outcomes"])


def _zcircuit():
    c = C.linear_cluster(5)
    c[2] = C.Ment("Z")
    return c


def test_z_sample_mode_matches_oracle_with_the_drawn_outcomes():
    """Sample mode: the kernel draws each Z outcome (SplitMix64 of seed, run,
    step); with those outcomes forced, the oracle gives the same state."""
    rng = np.random.default_rng(41)
    circ = _zcircuit()
    sw = DensityMatrixSweep(circ)
    B = 64
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    inp = haar_states(rng, 1, B)
    rho, outc, status, _ = sw.forward(ang, inp, seed=1234)
    rho2, outc2, _, _ = sw.forward(ang, inp, seed=1234)
    rho3, outc3, _, _ = sw.forward(ang, inp, seed=99)
    torch.cuda.synchronize()
    assert (status.cpu().numpy() == 0).all()
    assert torch.equal(outc, outc2) and torch.equal(rho, rho2)  # reproducible per seed
    zk = sw.plan.schedule_measure.index(2)
    assert not torch.equal(outc[:, zk], outc3[:, zk])  # and drawn
    outc = outc.cpu().numpy()
    rho = rho.cpu().numpy()
    for r in range(B):
        ref, ref_out, _ = oracle.run_dm(circ, ang[r], inp[r], z_outcomes={2: int(outc[r][zk])})
        assert np.abs(rho[r] - ref).max() < TOL_RHO_C64
        assert [ref_out[n] for n in sw.plan.schedule_measure] == list(outc[r])


def test_z_sample_mode_outcome_frequencies():
    rng = np.random.default_rng(43)
    circ = _zcircuit()
    sw = DensityMatrixSweep(circ)
    ang = rng.uniform(0, 2 * np.pi, size=sw.n_angles)
    inp = haar_states(rng, 1, 1)[0]
    B = 20000
    _, outc, status, _ = sw.forward(np.tile(ang, (B, 1)), inp, seed=7)
    torch.cuda.synchronize()
    zk = sw.plan.schedule_measure.index(2)
    frac1 = float(outc[:, zk].float().mean())
    # prob1 / (prob0 + prob1) at the Z step, from the oracle in expectation mode
    _, ref_out, _ = oracle.run_dm(circ, ang, inp, mode="expectation")
    p1 = ref_out[2]
    assert abs(frac1 - p1) < 5 * np.sqrt(p1 * (1 - p1) / B) + 1e-3


def test_z_expectation_through_the_simulator_and_rejections():
    from mentpy_gb300 import _native

    circ = _zcircuit()
    spec, data = load_golden("dm_zexp_lin5")
    sim = PatternSimulator(circuit_from_spec(spec), backend="cuda-dm")
    sim.reset(input_state=data["inputs"][0])
    rho = sim.run(data["angles"][0], mode="expectation")
    assert np.abs(rho - data["dm_rho"][0]).max() < TOL_RHO_C64
    vals = list(sim.outcomes.values())
    assert isinstance(vals[2], float) and abs(vals[2] - data["dm_zexp_outcomes"][0][2]) < 1e-5
    # the adjoint declines Z-basis circuits; the statevector sweep rejects them like the reference
    sw = DensityMatrixSweep(circ)
    with pytest.raises(_native.MbqcError):
        sw.adjoint(np.zeros((1, sw.n_angles)), None, np.zeros((1, 2, 2), dtype=np.complex64))
    with pytest.raises(ValueError, match="only XY plane"):
        compile_plan(circ, "sv")


def test_run_batch_on_the_dropin_density_matrix_simulator():
    circ = C.grid_cluster(3, 4)
    rng = np.random.default_rng(62)
    B = 40
    ang = rng.uniform(0, 2 * np.pi, size=(B, len(circ.trainable_nodes)))
    psi = haar_states(rng, 3, B)
    ps = PatternSimulator(circ, backend="cuda-dm", noise=0.01)
    rho, outc, status, probs = ps.run_batch(ang, psi)
    ref, ref_out, ref_probs = oracle.run_dm_batch(circ, ang, psi, noise_p=0.01)
    assert (status == 0).all()
    assert np.abs(rho - ref).max() < TOL_RHO_C64
    assert np.array_equal(outc, ref_out)
    assert np.abs(probs - ref_probs).max() < 1e-5
    ps.reset(input_state=psi[3])
    assert np.abs(ps.run(ang[3]) - rho[3]).max() < 1e-6


@pytest.mark.parametrize("noise", [0.0, 0.01])
def test_window_8_density_matrix(noise):
    """Window 8 (256 x 256 density matrix): the factored kernel keeps the
    128 x 128 matrix of the other bits in shared memory."""
    circ = C.many_wires([5] * 7)
    sw = DensityMatrixSweep(circ)
    assert sw.plan.window == 8
    rng = np.random.default_rng(71)
    B = 6
    ang = rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles))
    psi = haar_states(rng, 7, B)
    rho, outc, st, probs = sw.forward(ang, psi, noise=noise, want_probs=True)
    assert (st.cpu().numpy() == 0).all()
    ref, ref_out, ref_probs = oracle.run_dm_batch(circ, ang, psi, noise_p=noise)
    assert np.abs(rho.cpu().numpy() - ref).max() < TOL_RHO_C64
    assert np.array_equal(outc.cpu().numpy(), ref_out)
    assert np.abs(probs.cpu().numpy() - ref_probs).max() < 1e-5


def test_factored_and_full_matrix_kernels_agree():
    """The factored kernel (default) and the full-matrix kernel give the same
    states to float rounding and the same outcome bits on every window they
    share."""
    rng = np.random.default_rng(72)
    for circ in (C.many_wires([6] * 2), C.many_wires([5] * 3), C.grid_cluster(4, 3), C.many_wires([6] * 5),
                 C.many_wires([7] * 6)):
        sw = DensityMatrixSweep(circ)
        ang = rng.uniform(-9, 9, size=(33, sw.n_angles))
        psi = haar_states(rng, sw.n_in, 33)
        a = sw.forward(ang, psi, noise=0.02, want_probs=True)
        b = sw.forward(ang, psi, noise=0.02, want_probs=True, full_matrix=True)
        assert (a[2] == 0).all() and (b[2] == 0).all()
        assert (a[0] - b[0]).abs().max().item() < 1e-5
        assert torch.equal(a[1], b[1])
        assert (a[3] - b[3]).abs().max().item() < 1e-6


def test_persistent_batch_equals_per_window_launches_and_tunes():
    """One persistent launch over the uneven table gives the results of one
    launch per window size (same per-run arithmetic and tile shapes);
    after autotuning the tile shapes it still matches the oracle, and a
    captured graph replays it."""
    from mentpy_gb300.native_plan import GraphBatch

    rng = np.random.default_rng(73)
    shapes = [(int(rng.integers(2, 8)), int(rng.integers(3, 13))) for _ in range(300)]
    per = UnevenDensityMatrixBatch.from_graph_batch(GraphBatch.many_wires(shapes))
    per.persistent = False
    pers = UnevenDensityMatrixBatch.from_graph_batch(GraphBatch.many_wires(shapes))
    assert pers.persistent
    b1, b2 = per.allocate(), pers.allocate()
    angs, psis = [], []
    for c, p in enumerate(per.plans):
        a = rng.uniform(0, 2 * np.pi, p.n_angles)
        v = haar_states(rng, p.n_in, 1)[0]
        angs.append(a)
        psis.append(v)
        for b in (b1, b2):
            b["angles"][c, : p.n_angles] = torch.as_tensor(a)
            b["inputs"][c, : 2 ** p.n_in] = torch.as_tensor(v, dtype=torch.complex64)
    per.run(b1, noise=0.01)
    pers.run(b2, noise=0.01)
    torch.cuda.synchronize()
    assert int((b2["status"] != 0).sum()) == 0
    # the same per-run arithmetic (separately compiled kernels may contract
    # float operations differently: equal to rounding, outcome bits exact)
    assert (b1["rho"] - b2["rho"]).abs().max().item() < 1e-6
    assert torch.equal(b1["outcomes"], b2["outcomes"])
    # the longest circuits of windows 6 and 7 in their own tile shape
    assert 7 in pers.long_steps and 6 in pers.long_steps
    pers.long_tpr, pers._nbatch = {6: 128, 7: 256}, None
    b2["rho"].zero_()
    pers.run(b2, noise=0.01)
    torch.cuda.synchronize()
    assert int((b2["status"] != 0).sum()) == 0
    assert (b1["rho"] - b2["rho"]).abs().max().item() < 1e-6
    assert torch.equal(b1["outcomes"], b2["outcomes"])
    info = pers.tune(b2, noise=0.01, reps=2)
    assert info["candidates"] >= 2 and "long_circuit_tile_threads" in info
    b2["rho"].zero_()
    pers.capture(b2, noise=0.01)
    b2["rho"].zero_()
    pers.run(b2, noise=0.01)  # graph replay of the tuned launch
    pers.run(b2, noise=0.01)  # the claim counter was reset by the previous launch
    torch.cuda.synchronize()
    assert int((b2["status"] != 0).sum()) == 0
    for c in rng.choice(len(shapes), 40, replace=False):
        W, D = shapes[c]
        ref, outc, _ = oracle.run_dm(C.many_wires([D] * W), angs[c], psis[c], noise_p=0.01)
        assert np.abs(pers.rho(b2, c).cpu().numpy() - ref).max() < TOL_RHO_C64
        M = pers.plans[c].n_steps
        assert list(b2["outcomes"][c, :M].cpu().numpy()) == list(outc.values())


@pytest.mark.parametrize("build,B,noise", [(lambda: C.many_wires([4] * 8), 4, 0.01),
                                           (lambda: C.grid_cluster(9, 3), 2, 0.02)])
def test_wide_window_density_matrix_against_oracle(build, B, noise):
    """Windows 9 and 10: the factored matrix (512 KB, 2 MB per run) lives in a
    device workspace, one 1024-thread block per run; the reference runs these
    windows with dense operators (np_simulator_dm.py:33-346)."""
    circ = build()
    sw = DensityMatrixSweep(circ)
    assert sw.plan.window in (9, 10)
    rng = np.random.default_rng(74)
    ang = rng.uniform(-50, 50, size=(B, sw.n_angles))
    psi = haar_states(rng, sw.n_in, B)
    rho, outc, st, probs = sw.forward(ang, psi, noise=noise, want_probs=True)
    assert (st.cpu().numpy() == 0).all()
    ref, ref_out, ref_probs = oracle.run_dm_batch(circ, ang, psi, noise_p=noise)
    assert np.abs(rho.cpu().numpy() - ref).max() < TOL_RHO_C64
    assert np.array_equal(outc.cpu().numpy(), ref_out)
    assert np.abs(probs.cpu().numpy() - ref_probs).max() < 1e-5


def test_window_11_density_matrix_equals_statevector_and_dropin():
    """Window 11 (an 8 MB factored matrix per run): without noise the density
    matrix is the outer product of the statevector sweep's output, through
    the drop-in PatternSimulator(backend="cuda-dm") as well."""
    from mentpy_gb300.sweep import StatevectorSweep

    circ = C.grid_cluster(10, 3)
    rng = np.random.default_rng(75)
    ang = rng.uniform(0, 2 * np.pi, size=(2, len(circ.trainable_nodes)))
    psi = haar_states(rng, 10, 2)
    sw = DensityMatrixSweep(circ)
    assert sw.plan.window == 11
    rho, _, st, _ = sw.forward(ang, psi)
    sv, sst, _ = StatevectorSweep(circ).forward(ang, psi)
    assert (st.cpu().numpy() == 0).all() and (sst.cpu().numpy() == 0).all()
    ref = torch.einsum("bi,bj->bij", sv, sv.conj())
    assert (rho - ref).abs().max().item() < 2e-5
    ps = PatternSimulator(circ, backend="cuda-dm")
    ps.reset(input_state=psi[1])
    assert np.abs(ps.run(ang[1]) - ref[1].cpu().numpy()).max() < 2e-5
