"""Native plan compilation: open graphs to window plans in C++.

``compile_plan_native(circuit, kind)`` gives the same ``WindowPlan`` as
``plan.compile_plan`` (which restates the reference's constructors in
Python), computed by ``mbqc_compile_graph`` in libmbqc_gb300: causal-flow
layers, measurement order and window tables without networkx.  Where the
native compiler declines (no causal flow, measured outputs, a flow search
whose result depends on Python's set iteration order, an explicit schedule)
the Python compiler runs instead, so results and error messages always match
the reference's.

``compile_graph_plans`` compiles raw open graphs (node, edge and measurement
arrays, no ``MBQCircuit``) -- the path for batches of thousands of uneven
circuits, where building networkx circuits in Python dominates.
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy as np

from . import _native
from .plan import PLANE_CODES, WindowPlan, compile_plan

__all__ = ["compile_plan_native", "compile_graph_plans", "compile_graph_batch", "GraphSpec", "GraphBatch",
           "PlanInfo", "many_wires_spec"]


class GraphSpec:
    """An open graph with measurements as flat arrays.

    ``nodes``: labels in graph order; ``edges``: [E, 2] labels; ``planes``:
    per node a key of ``PLANE_CODES`` or None (outputs); ``angles``: per node
    a float or None (trainable).  ``trainable_order``: labels in angle-vector
    order (default: graph order of the trainable nodes).
    """

    def __init__(self, nodes, edges, inputs, outputs, planes, angles, trainable_order=None):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        self.edges = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1, 2))
        self.inputs = np.ascontiguousarray(inputs, dtype=np.int32)
        self.outputs = np.ascontiguousarray(outputs, dtype=np.int32)
        self.plane = np.array([-1 if p is None else PLANE_CODES[p] for p in planes], dtype=np.int32)
        self.trainable = np.array([1 if (p is not None and a is None) else 0 for p, a in zip(planes, angles)],
                                  dtype=np.int32)
        self.angle = np.array([0.0 if a is None else float(a) for a in angles], dtype=np.float64)
        self.trainable_order = (None if trainable_order is None
                                else np.ascontiguousarray(trainable_order, dtype=np.int32))

    @classmethod
    def from_circuit(cls, circuit) -> "GraphSpec":
        g = circuit.graph
        nodes = list(g.nodes)
        planes, angles = [], []
        for v in nodes:
            m = circuit[v]
            planes.append(None if m is None else m.plane)
            angles.append(None if (m is None or m.angle is None) else m.angle)
        return cls(nodes, list(g.edges), list(circuit.input_nodes), list(circuit.output_nodes), planes, angles,
                   trainable_order=list(circuit.trainable_nodes))


def _ptr(a, ctype):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctype))


def _compile_spec(spec: GraphSpec, kind: str, window_size: int):
    """(rc, WindowPlan or None) from the native compiler."""
    n = len(spec.nodes)
    d = _native.GraphDesc()
    d.n_nodes = n
    d.nodes = _ptr(spec.nodes, ctypes.c_int32)
    d.n_edges = len(spec.edges)
    d.edges = _ptr(spec.edges, ctypes.c_int32)
    d.n_inputs = len(spec.inputs)
    d.inputs = _ptr(spec.inputs, ctypes.c_int32)
    d.n_outputs = len(spec.outputs)
    d.outputs = _ptr(spec.outputs, ctypes.c_int32)
    d.plane = _ptr(spec.plane, ctypes.c_int32)
    d.trainable = _ptr(spec.trainable, ctypes.c_int32)
    d.angle = _ptr(spec.angle, ctypes.c_double)
    d.n_trainable = 0 if spec.trainable_order is None else len(spec.trainable_order)
    d.trainable_order = _ptr(spec.trainable_order, ctypes.c_int32)
    d.window_size = int(window_size)
    d.kind = 0 if kind == "sv" else 1
    cap = max(n, 1)
    arr = dict(in_bits=np.zeros(cap, np.int32), init_cz=np.zeros(32, np.uint32), step_mask=np.zeros(cap, np.uint32),
               step_angle=np.zeros(cap, np.int32), step_plane=np.zeros(cap, np.int32),
               step_fixed_angle=np.zeros(cap, np.float64), out_bits=np.zeros(cap, np.int32),
               out_nodes=np.zeros(cap, np.int32), schedule=np.zeros(cap, np.int32))
    t = _native.PlanTables()
    t.in_bits = _ptr(arr["in_bits"], ctypes.c_int32)
    t.init_cz = _ptr(arr["init_cz"], ctypes.c_uint32)
    t.step_mask = _ptr(arr["step_mask"], ctypes.c_uint32)
    t.step_angle = _ptr(arr["step_angle"], ctypes.c_int32)
    t.step_plane = _ptr(arr["step_plane"], ctypes.c_int32)
    t.step_fixed_angle = _ptr(arr["step_fixed_angle"], ctypes.c_double)
    t.out_bits = _ptr(arr["out_bits"], ctypes.c_int32)
    t.out_nodes = _ptr(arr["out_nodes"], ctypes.c_int32)
    t.schedule = _ptr(arr["schedule"], ctypes.c_int32)
    rc = _native.lib().mbqc_compile_graph(ctypes.byref(d), ctypes.byref(t))
    if rc != _native.MBQC_OK:
        return rc, None
    w, M, n_in, n_out, A = t.window, t.n_steps, t.n_in, t.n_out, t.n_angles
    schedule = [int(x) for x in arr["schedule"][:n]]
    out_set = set(int(x) for x in spec.outputs)
    sched_meas = [v for v in schedule if v not in out_set][:M]
    if spec.trainable_order is not None:
        trainable = [int(x) for x in spec.trainable_order]
    else:
        trainable = [int(v) for v, tr in zip(spec.nodes, spec.trainable) if tr]
    plan = WindowPlan(
        kind=kind, window=w, n_nodes=n, schedule=schedule, schedule_measure=sched_meas, n_in=n_in, n_out=n_out,
        n_angles=A, trainable_nodes=trainable, in_bits=arr["in_bits"][:n_in].copy(),
        init_cz=arr["init_cz"][:w].copy(), step_mask=arr["step_mask"][:M].copy(),
        step_angle=arr["step_angle"][:M].copy(), step_plane=arr["step_plane"][:M].copy(),
        step_fixed_angle=arr["step_fixed_angle"][:M].copy(), out_bits=arr["out_bits"][:n_out].copy(),
        out_nodes=[int(x) for x in arr["out_nodes"][:n_out]], output_ment_nodes=[])
    return rc, plan


def compile_plan_native(circuit, kind: str = "sv", window_size: int = 1, schedule=None, force0: bool = True,
                        dev_mode: bool = False) -> WindowPlan:
    """``compile_plan`` through the native compiler, with the Python compiler
    as the fallback for what the native one declines."""
    if schedule is not None or not force0 or dev_mode or kind not in ("sv", "dm"):
        return compile_plan(circuit, kind, window_size=window_size, schedule=schedule, force0=force0,
                            dev_mode=dev_mode)
    try:
        spec = GraphSpec.from_circuit(circuit)
    except (KeyError, TypeError, ValueError):
        return compile_plan(circuit, kind, window_size=window_size)
    rc, plan = _compile_spec(spec, kind, window_size)
    if plan is None:
        return compile_plan(circuit, kind, window_size=window_size)
    return plan


def compile_graph_plans(specs: Sequence[GraphSpec], kind: str = "dm", window_size: int = 1) -> List[WindowPlan]:
    """Native plans of many raw open graphs.  Raises ``ValueError`` naming the
    first graph the native compiler declines (build an ``MBQCircuit`` and use
    ``compile_plan`` for those)."""
    out = []
    for i, spec in enumerate(specs):
        rc, plan = _compile_spec(spec, kind, window_size)
        if plan is None:
            msg = _native.lib().mbqc_last_error()
            raise ValueError(f"graph {i}: {msg.decode() if msg else rc}")
        out.append(plan)
    return out


def many_wires_spec(depths: Sequence[int]) -> GraphSpec:
    """The open graph of ``templates.many_wires(depths)`` as a ``GraphSpec``
    (wire i is a path of depths[i] nodes, input at its start, output at its
    end, all measured nodes trainable XY), without building an MBQCircuit."""
    nodes, edges, inputs, outputs = [], [], [], []
    base = 0
    for d in depths:
        if d < 2:
            raise ValueError("each wire needs at least two nodes")
        wire = list(range(base, base + d))
        nodes += wire
        edges += [(wire[i], wire[i + 1]) for i in range(d - 1)]
        inputs.append(wire[0])
        outputs.append(wire[-1])
        base += d
    out_set = set(outputs)
    planes = [None if v in out_set else "XY" for v in nodes]
    angles = [None] * len(nodes)
    return GraphSpec(nodes, edges, inputs, outputs, planes, angles)


class PlanInfo:
    """Shape of one natively compiled plan (what batch launchers need)."""

    __slots__ = ("kind", "window", "n_steps", "n_in", "n_out", "n_angles", "n_nodes")

    def __init__(self, kind, window, n_steps, n_in, n_out, n_angles, n_nodes):
        self.kind, self.window, self.n_steps = kind, int(window), int(n_steps)
        self.n_in, self.n_out, self.n_angles, self.n_nodes = int(n_in), int(n_out), int(n_angles), int(n_nodes)


class GraphBatch:
    """Many open graphs in flat arrays (graph i owns entries
    ``[off[i], off[i+1])``; every trainable angle in graph order)."""

    def __init__(self, node_off, nodes, plane, trainable, angle, edge_off, edges, in_off, inputs, out_off,
                 outputs):
        i64 = lambda a: np.ascontiguousarray(a, dtype=np.int64)  # noqa: E731
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
        self.node_off, self.edge_off, self.in_off, self.out_off = (i64(node_off), i64(edge_off), i64(in_off),
                                                                   i64(out_off))
        self.nodes, self.plane, self.trainable = i32(nodes), i32(plane), i32(trainable)
        self.angle = np.ascontiguousarray(angle, dtype=np.float64)
        self.edges = i32(np.asarray(edges).reshape(-1, 2)) if len(edges) else np.zeros((0, 2), np.int32)
        self.inputs, self.outputs = i32(inputs), i32(outputs)

    @property
    def n_graphs(self) -> int:
        return len(self.node_off) - 1

    @classmethod
    def from_specs(cls, specs: Sequence[GraphSpec]) -> "GraphBatch":
        cat = lambda xs, dt: np.concatenate(xs).astype(dt) if len(xs) else np.zeros(0, dt)  # noqa: E731
        off = lambda xs: np.concatenate([[0], np.cumsum([len(x) for x in xs])])  # noqa: E731
        for sp in specs:
            if sp.trainable_order is not None and list(sp.trainable_order) != [
                    int(v) for v, t in zip(sp.nodes, sp.trainable) if t]:
                raise ValueError("graph batches take angles in graph order")
        return cls(off([s.nodes for s in specs]), cat([s.nodes for s in specs], np.int32),
                   cat([s.plane for s in specs], np.int32), cat([s.trainable for s in specs], np.int32),
                   cat([s.angle for s in specs], np.float64), off([s.edges for s in specs]),
                   np.concatenate([s.edges for s in specs]) if specs else np.zeros((0, 2)),
                   off([s.inputs for s in specs]), cat([s.inputs for s in specs], np.int32),
                   off([s.outputs for s in specs]), cat([s.outputs for s in specs], np.int32))

    @classmethod
    def many_wires(cls, shapes: Sequence[Sequence[int]]) -> "GraphBatch":
        """``many_wires([D] * W)`` for every (W, D) in ``shapes``, vectorised."""
        W = np.asarray([s[0] for s in shapes], dtype=np.int64)
        D = np.asarray([s[1] for s in shapes], dtype=np.int64)
        if (W < 1).any() or (D < 2).any():
            raise ValueError("wires need at least two nodes")
        n = W * D
        node_off = np.concatenate([[0], np.cumsum(n)])
        g_of_node = np.repeat(np.arange(len(W)), n)
        local = np.arange(node_off[-1]) - node_off[g_of_node]
        Dn = D[g_of_node]
        is_out = (local % Dn) == Dn - 1
        ne = W * (D - 1)
        edge_off = np.concatenate([[0], np.cumsum(ne)])
        g_of_edge = np.repeat(np.arange(len(W)), ne)
        le = np.arange(edge_off[-1]) - edge_off[g_of_edge]
        De = D[g_of_edge]
        a = (le // (De - 1)) * De + le % (De - 1)
        io_off = np.concatenate([[0], np.cumsum(W)])
        g_of_io = np.repeat(np.arange(len(W)), W)
        wire = np.arange(io_off[-1]) - io_off[g_of_io]
        starts = wire * D[g_of_io]
        return cls(node_off, local, np.where(is_out, -1, PLANE_CODES["XY"]), (~is_out).astype(np.int32),
                   np.zeros(node_off[-1]), edge_off, np.stack([a, a + 1], axis=1), io_off, starts, io_off,
                   starts + D[g_of_io] - 1)

    def _desc(self, kind: str, window_size: int):
        d = _native.GraphBatchDesc()
        d.n_graphs = self.n_graphs
        d.node_off = _ptr(self.node_off, ctypes.c_int64)
        d.nodes = _ptr(self.nodes, ctypes.c_int32)
        d.plane = _ptr(self.plane, ctypes.c_int32)
        d.trainable = _ptr(self.trainable, ctypes.c_int32)
        d.angle = _ptr(self.angle, ctypes.c_double)
        d.edge_off = _ptr(self.edge_off, ctypes.c_int64)
        d.edges = _ptr(self.edges, ctypes.c_int32)
        d.in_off = _ptr(self.in_off, ctypes.c_int64)
        d.inputs = _ptr(self.inputs, ctypes.c_int32)
        d.out_off = _ptr(self.out_off, ctypes.c_int64)
        d.outputs = _ptr(self.outputs, ctypes.c_int32)
        d.window_size = int(window_size)
        d.kind = 0 if kind == "sv" else 1
        return d


def compile_graph_batch(batch: GraphBatch, kind: str = "dm", window_size: int = 1, upload: bool = True):
    """Compile every graph of ``batch`` natively.  Returns ``(device_plan,
    infos)``: a ``DevicePlan`` holding all circuits (circuit i = graph i; None
    with ``upload=False``, which needs no GPU) and one ``PlanInfo`` each."""
    d = batch._desc(kind, window_size)
    info = np.zeros((batch.n_graphs, 5), dtype=np.int32)
    h = ctypes.c_void_p()
    rc = _native.lib().mbqc_plan_create_from_graphs(ctypes.byref(d), ctypes.byref(h) if upload else None,
                                                    info.ctypes.data_as(ctypes.c_void_p))
    if rc != _native.MBQC_OK:
        msg = _native.lib().mbqc_last_error()
        raise ValueError(msg.decode() if msg else f"native compile failed ({rc})")
    nn = np.diff(batch.node_off)
    infos = [PlanInfo(kind, *row, n_nodes) for row, n_nodes in zip(info.tolist(), nn.tolist())]
    dplan = _native.DevicePlan.from_handle(h, infos) if upload else None
    return dplan, infos
