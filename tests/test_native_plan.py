"""Native plan compiler (host code, no GPU) against the Python compiler.

Every plan table must be identical to ``compile_plan``'s (which is pinned to
the reference by the golden fixtures), or the native compiler must decline
and the Python compiler run instead.
"""
import numpy as np
import pytest

from mentpy_gb300 import _native
from mentpy_gb300 import circuit as C
from mentpy_gb300.native_plan import (GraphSpec, _compile_spec, compile_graph_plans, compile_plan_native,
                                      many_wires_spec)
from mentpy_gb300.plan import compile_plan



@pytest.fixture(scope="module", autouse=True)
def _library():
    from mentpy_gb300 import build

    build.build()

FIELDS_ARR = ["in_bits", "init_cz", "step_mask", "step_angle", "step_plane", "step_fixed_angle", "out_bits"]
FIELDS = ["kind", "window", "n_nodes", "schedule", "schedule_measure", "n_in", "n_out", "n_angles",
          "trainable_nodes", "out_nodes", "output_ment_nodes"]


def assert_same_plan(a, b):
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), f
    for f in FIELDS_ARR:
        x, y = getattr(a, f), getattr(b, f)
        assert x.dtype == y.dtype and np.array_equal(x, y), f


def _circuits():
    cs = [C.linear_cluster(n) for n in (3, 4, 7, 12)]
    cs += [C.many_wires(list(d)) for d in ([2, 3], [8] * 4, [12] * 6, [3, 9, 5], [4, 4, 4, 4, 4, 4])]
    cs += [C.grid_cluster(r, c) for r, c in ((2, 3), (3, 4), (4, 4), (6, 4), (16, 10))]
    cs += [C.muta(2, 1), C.muta(3, 1), C.muta(2, 2)]
    cs += [C.hstack((C.many_wires([3, 3]), C.grid_cluster(2, 4)))]
    return cs


@pytest.mark.parametrize("kind", ["sv", "dm"])
def test_native_plans_equal_python_plans(kind):
    declined = 0
    for circ in _circuits():
        try:
            want = compile_plan(circ, kind)
        except (ValueError, NotImplementedError):
            continue
        rc, got = _compile_spec(GraphSpec.from_circuit(circ), kind, 1)
        if got is None:
            declined += 1
            assert rc == _native.MBQC_E_UNSUPPORTED
            continue
        assert_same_plan(got, want)
    assert declined <= 3


def test_random_graphs_equal_or_declined():
    rng = np.random.default_rng(3)
    n_same = n_declined = 0
    for trial in range(60):
        depths = [int(x) for x in rng.integers(2, 7, size=int(rng.integers(1, 5)))]
        circ = C.many_wires(depths)
        # a few random cross-wire edges (rebuilds the circuit; skip when no flow)
        for _ in range(int(rng.integers(0, 4))):
            u, v = (int(x) for x in rng.integers(0, sum(depths), size=2))
            if u == v:
                continue
            try:
                circ.add_edge(u, v)
            except ValueError:
                pass
        if circ.measurement_order is None:
            continue
        for kind in ("sv", "dm"):
            try:
                want = compile_plan(circ, kind)
            except (ValueError, NotImplementedError):
                continue
            rc, got = _compile_spec(GraphSpec.from_circuit(circ), kind, 1)
            if got is None:
                n_declined += 1
                continue
            assert_same_plan(got, want)
            n_same += 1
    assert n_same > 40


def test_compile_plan_native_falls_back_to_python():
    circ = C.many_wires([4, 4])
    assert_same_plan(compile_plan_native(circ, "sv"), compile_plan(circ, "sv"))
    # explicit schedule: always the Python compiler
    sched = list(circ.measurement_order)
    assert_same_plan(compile_plan_native(circ, "sv", schedule=sched, window_size=3),
                     compile_plan(circ, "sv", schedule=sched, window_size=3))
    # Python errors come through unchanged
    with pytest.raises(ValueError, match="Window size is set to 9"):
        compile_plan_native(circ, "sv", window_size=9)


def test_many_wires_spec_matches_template():
    rng = np.random.default_rng(5)
    for _ in range(20):
        depths = [int(x) for x in rng.integers(2, 13, size=int(rng.integers(2, 7)))]
        want = compile_plan(C.many_wires(depths), "dm")
        (got,) = compile_graph_plans([many_wires_spec(depths)], "dm")
        assert_same_plan(got, want)


def test_declines_are_reported():
    # a graph without causal flow: two inputs/outputs, one shared middle node
    spec = GraphSpec([0, 1, 2, 3, 4], [(0, 2), (1, 2), (2, 3), (2, 4)], [0, 1], [3, 4],
                     ["XY", "XY", "XY", None, None], [None] * 5)
    rc, plan = _compile_spec(spec, "dm", 1)
    assert plan is None and rc == _native.MBQC_E_UNSUPPORTED
    with pytest.raises(ValueError, match="graph 0"):
        compile_graph_plans([spec], "dm")


def test_graph_batch_compile_only_matches_python_plans():
    from mentpy_gb300.native_plan import GraphBatch, compile_graph_batch

    rng = np.random.default_rng(9)
    shapes = [(int(rng.integers(1, 7)), int(rng.integers(2, 13))) for _ in range(64)]
    shapes = [(w, d) for w, d in shapes if w * (d - 1) >= w + 1]  # enough measurements for the window
    batch = GraphBatch.many_wires(shapes)
    ref = GraphBatch.from_specs([many_wires_spec([d] * w) for w, d in shapes])
    for k in ("node_off", "nodes", "plane", "trainable", "angle", "edge_off", "edges", "in_off", "inputs",
              "out_off", "outputs"):
        assert np.array_equal(getattr(batch, k), getattr(ref, k)), k
    dplan, infos = compile_graph_batch(batch, "dm", upload=False)
    assert dplan is None and len(infos) == len(shapes)
    for (w, d), info in zip(shapes, infos):
        p = compile_plan(C.many_wires([d] * w), "dm")
        assert (info.window, info.n_steps, info.n_in, info.n_out, info.n_angles, info.n_nodes) == (
            p.window, p.n_steps, p.n_in, p.n_out, p.n_angles, p.n_nodes)


def test_graph_batch_names_the_declined_graph():
    from mentpy_gb300.native_plan import GraphBatch, compile_graph_batch

    bad = GraphSpec([0, 1, 2, 3, 4], [(0, 2), (1, 2), (2, 3), (2, 4)], [0, 1], [3, 4],
                    ["XY", "XY", "XY", None, None], [None] * 5)
    batch = GraphBatch.from_specs([many_wires_spec([4, 4]), bad])
    with pytest.raises(ValueError, match="graph 1"):
        compile_graph_batch(batch, "dm", upload=False)
