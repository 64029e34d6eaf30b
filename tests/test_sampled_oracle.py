"""The restated PennyLane circuit with byproduct corrections (CPU): with every
outcome 0 it is the reference's force0 sweep (pinned by the fixtures through
the windowed oracle); with any outcomes the corrections make the output the
same state up to a global phase (causal-flow determinism)."""
import numpy as np
import pytest

from helpers import haar_states
from mentpy_gb300 import circuit as C
from mentpy_gb300.plan import compile_plan
from mentpy_gb300.sampling import byproduct_tables
from oracle import fullcircuit, sweep


def _infid(a, b):
    return 1.0 - abs(np.vdot(a / np.linalg.norm(a), b / np.linalg.norm(b))) ** 2


# circuits whose default window holds every CZ partner of a node before it is
# measured (there the windowed sweep is the whole-graph circuit; for e.g.
# many_wires([3, 4]) the reference's default window drops a CZ and differs)
@pytest.mark.parametrize("build", [lambda: C.linear_cluster(6), lambda: C.many_wires([3, 3]),
                                   lambda: C.grid_cluster(2, 4), lambda: C.grid_cluster(3, 3)])
def test_corrected_circuit_is_outcome_independent(build):
    circ = build()
    plan = compile_plan(circ, "sv")
    rng = np.random.default_rng(61)
    ang = rng.uniform(0, 2 * np.pi, len(circ.trainable_nodes))
    inp = haar_states(rng, len(circ.input_nodes), 1)[0]
    zero = {v: 0 for v in plan.schedule_measure}
    base = fullcircuit.run_full_sampled_sv(circ, ang, inp, zero, plan.out_nodes)
    ref = sweep.run_sv(circ, ang, inp, output_form="sv")[0]
    assert _infid(base, ref) < 1e-12
    for _ in range(6):
        oc = {v: int(rng.integers(0, 2)) for v in plan.schedule_measure}
        out = fullcircuit.run_full_sampled_sv(circ, ang, inp, oc, plan.out_nodes)
        assert _infid(out, base) < 1e-12


@pytest.mark.parametrize("build", [lambda: C.linear_cluster(6), lambda: C.many_wires([3, 3]),
                                   lambda: C.grid_cluster(2, 4), lambda: C.grid_cluster(3, 3)])
def test_windowed_sampled_oracle_matches_whole_circuit(build):
    """The windowed restatement of the corrected circuit (gates in the window,
    deferred Z on nodes not yet added) against the whole-graph circuit, for
    random outcomes."""
    circ = build()
    plan = compile_plan(circ, "sv")
    rng = np.random.default_rng(62)
    ang = rng.uniform(0, 2 * np.pi, len(circ.trainable_nodes))
    inp = haar_states(rng, len(circ.input_nodes), 1)[0]
    for _ in range(6):
        oc = {v: int(rng.integers(0, 2)) for v in plan.schedule_measure}
        full = fullcircuit.run_full_sampled_sv(circ, ang, inp, oc, plan.out_nodes)
        win = sweep.run_sv_sampled(circ, ang, inp, oc)
        assert _infid(win, full) < 1e-12


def test_windowed_sampled_oracle_long_sweep():
    """Outcome independence through the window on a sweep of 238 steps (the
    whole-graph circuit cannot run there)."""
    circ = C.many_wires([120, 120])
    plan = compile_plan(circ, "sv")
    rng = np.random.default_rng(63)
    ang = rng.uniform(0, 2 * np.pi, len(circ.trainable_nodes))
    inp = haar_states(rng, 2, 1)[0]
    base = sweep.run_sv(circ, ang, inp, output_form="sv")[0]
    oc = {v: int(rng.integers(0, 2)) for v in plan.schedule_measure}
    assert _infid(sweep.run_sv_sampled(circ, ang, inp, oc), base) < 1e-10


def test_byproduct_tables_follow_the_flow():
    circ = C.linear_cluster(5)
    plan = compile_plan(circ, "sv")
    xs, zoff, zidx, xo, zo = byproduct_tables(circ, plan)
    # 0 -> 1 -> 2 -> 3 -> 4 (output): X on the successor, Z on the node after it
    assert list(xs) == [1, 2, 3, -1]
    assert int(xo[3]) == 1 and not xo[:3].any()
    assert list(zoff) == [0, 1, 2, 2, 2] and list(zidx) == [2, 3]
    assert int(zo[2]) == 1 and int(zo[3]) == 0


def test_byproduct_tables_any_length():
    """No cap on the number of steps: a 400-step sweep gets one X target per
    step and Z targets only on later steps."""
    circ = C.many_wires([201, 201])
    plan = compile_plan(circ, "sv")
    xs, zoff, zidx, xo, zo = byproduct_tables(circ, plan)
    M = plan.n_steps
    assert M == 400 and len(zoff) == M + 1 and zoff[-1] == len(zidx)
    for k in range(M):
        assert xs[k] == -1 or xs[k] > k
        assert all(t > k for t in zidx[zoff[k]:zoff[k + 1]])


def _exec_plan_sv_frame(plan, tables, angles, psi_in, outc):
    """The sampled kernel's method in complex128 (no GPU): the force0 step of
    the plan tables with a Pauli frame instead of correction gates.  A pending
    X on step k conjugates its coefficient (angle -> -angle), a pending Z
    negates it (angle -> angle + pi); outcome 1 takes the other branch
    (coefficient -c); on outcome 1 the step's table entries toggle the frame
    of later steps and of the outputs, and the output frame permutes (X) and
    signs (Z) the output index at the end."""
    from helpers import DEAD, _initial_window, _out_index, _popc, _projector

    xs, zoff, zidx, xo_t, zo_t = (np.asarray(t) for t in tables)
    w, M = plan.window, plan.n_steps
    idx = np.arange(2**w)
    psi = _initial_window(plan, psi_in)
    fx, fz = np.zeros(M, bool), np.zeros(M, bool)
    xo = zo = 0
    for k in range(M):
        p = k % w
        a = int(plan.step_angle[k])
        theta = angles[a] if a >= 0 else plan.step_fixed_angle[k]
        P0, _ = _projector(int(plan.step_plane[k]), theta)
        c = (P0[1, 0] / P0[0, 0]).conjugate()  # phi = psi0 + c psi1 (<+_theta| up to a factor)
        if fx[k]:
            c = c.conjugate()
        if fz[k]:
            c = -c
        if outc[k]:
            c = -c
        lo = idx[((idx >> p) & 1) == 0]
        hi = lo | (1 << p)
        phi = psi[lo] + c * psi[hi]
        phi = phi / np.linalg.norm(phi)
        m = int(plan.step_mask[k])
        psi = psi.copy()
        psi[lo] = phi
        psi[hi] = 0 if m & DEAD else phi * np.where(_popc(hi & m) & 1, -1.0, 1.0)
        if outc[k]:
            if xs[k] > k:
                fx[xs[k]] ^= True
            for t in zidx[zoff[k]:zoff[k + 1]]:
                fz[t] ^= True
            xo ^= int(xo_t[k])
            zo ^= int(zo_t[k])
    y = np.arange(2**plan.n_out)
    out = np.zeros(2**plan.n_out, complex)
    yy = y ^ xo
    out[yy] = psi[_out_index(plan)] * np.where(_popc(yy & zo) & 1, -1.0, 1.0)
    return out / np.linalg.norm(out)


@pytest.mark.parametrize("build", [lambda: C.linear_cluster(7), lambda: C.many_wires([3, 3]),
                                   lambda: C.many_wires([6, 6, 6]), lambda: C.grid_cluster(2, 4),
                                   lambda: C.grid_cluster(3, 3), lambda: C.grid_cluster(4, 5)])
def test_frame_method_on_the_byproduct_tables_matches_the_corrected_circuit(build):
    """The sampled kernel's frame method, driven by sampling.byproduct_tables,
    gives the windowed oracle's corrected state for random outcomes."""
    circ = build()
    plan = compile_plan(circ, "sv")
    tables = byproduct_tables(circ, plan)
    rng = np.random.default_rng(64)
    ang = rng.uniform(0, 2 * np.pi, len(circ.trainable_nodes))
    inp = haar_states(rng, len(circ.input_nodes), 1)[0]
    for _ in range(4):
        outc = rng.integers(0, 2, plan.n_steps)
        oc = {v: int(o) for v, o in zip(plan.schedule_measure, outc)}
        ref = sweep.run_sv_sampled(circ, ang, inp, oc)
        got = _exec_plan_sv_frame(plan, tables, ang, inp, outc)
        assert _infid(got, ref) < 1e-12


def _fake(edges, order, flow, sched, outs, flow_none=False):
    """A circuit/plan pair carrying only what byproduct_tables reads."""
    import types

    import networkx as nx

    g = nx.Graph(edges)
    circ = types.SimpleNamespace(graph=g, measurement_order=order,
                                 flow=None if flow_none else (lambda v: flow[v]))
    plan = types.SimpleNamespace(n_steps=len(sched), n_out=len(outs), schedule_measure=sched, out_nodes=outs)
    return circ, plan


def test_byproduct_tables_error_paths():
    # no causal flow
    c, p = _fake([(0, 1)], [0, 1], {}, [0], [1], flow_none=True)
    with pytest.raises(ValueError, match="causal flow"):
        byproduct_tables(c, p)
    # more than 32 outputs (the frame is a 32-bit output mask)
    c, p = _fake([(0, 1)], [0, 1], {0: 1}, [0], list(range(1, 34)))
    with pytest.raises(ValueError, match="at most 32 output"):
        byproduct_tables(c, p)
    # flow(i) measured before i
    c, p = _fake([(0, 1), (1, 2)], [0, 1, 2], {0: 1, 1: 0}, [0, 1], [2])
    with pytest.raises(ValueError, match="measured before"):
        byproduct_tables(c, p)
    # flow(i) neither measured nor an output
    c, p = _fake([(0, 1), (0, 2)], [0, 1, 2], {0: 2}, [0], [1])
    with pytest.raises(ValueError, match="neither measured nor an output"):
        byproduct_tables(c, p)
    # a later-ordered neighbour of flow(i) that the window schedule measures first
    c, p = _fake([(0, 1), (1, 2), (2, 3)], [0, 1, 2, 3], {0: 2, 2: 3, 1: 3}, [1, 0, 2], [3])
    with pytest.raises(ValueError, match="in the window schedule"):
        byproduct_tables(c, p)
