"""Host-side MBQC circuit model: the source of every window plan.

This module restates, in its own code, the parts of mentpy's circuit layer that
decide *what* the windowed sweep does, so that the GPU backend can be driven
without mentpy installed:

* ``Ment``            -- measurement plane/angle, trainability and projector
                         (mentpy/operators/ment.py:123-260).
* ``MBQCircuit``      -- graph, input/output nodes, measurement dict, trainable
                         node order, quantum outputs, causal flow and the
                         measurement order (mentpy/mbqc/mbqcircuit.py:56-158,
                         325-373, 390-422).
* ``find_cflow``      -- causal flow, the published Mhalla--Perdrix algorithm
                         (arXiv:0709.2670) as used at mentpy/mbqc/flow.py:115-185.
* templates           -- ``linear_cluster``, ``many_wires``, ``grid_cluster``
                         and ``muta`` (mentpy/mbqc/templates.py:16-216) plus
                         ``hstack`` (mentpy/mbqc/mbqcircuit.py:519-611).

Every bookkeeping rule that changes the numbers the sweep produces is kept:
node iteration order (it fixes ``trainable_nodes``, the angle-vector layout),
the insertion order of the measurement dict, the set-iteration order of the
causal-flow search, and the tie-breaking of the measurement order.  The plan
compiler (``mentpy_gb300.plan``) also accepts mentpy's own ``MBQCircuit``
objects, which expose the same attributes.
"""
from __future__ import annotations

import copy
import math
import warnings
from functools import reduce
from typing import Callable, Dict, List, Optional

import numpy as np
import networkx as nx

__all__ = [
    "Ment",
    "Measurement",
    "GraphState",
    "MBQCircuit",
    "find_cflow",
    "hstack",
    "linear_cluster",
    "many_wires",
    "grid_cluster",
    "muta",
]

_PAULI_X = np.array([[0, 1], [1, 0]], dtype=complex)
_PAULI_Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
_PAULI_Z = np.array([[1, 0], [0, -1]], dtype=complex)

_PLANES = ("XY", "XZ", "YZ", "XYZ", "X", "Y", "Z")


class Ment:
    """A single-qubit measurement: a plane and an (optional, trainable) angle.

    Mirrors the constructor rules of mentpy's ``Ment``
    (mentpy/operators/ment.py:135-172): ``Ment("X")`` and ``Ment(0.3, "XY")``
    are both accepted, the Pauli planes carry angle 0, and a measurement is
    trainable exactly when it has no angle and a continuous plane
    (ment.py:214-216).
    """

    def __init__(self, angle=None, plane: Optional[str] = "XY"):
        if isinstance(angle, str):
            plane_arg = plane
            plane = angle
            angle = plane_arg if isinstance(plane_arg, (int, float, tuple)) else None
        elif not (isinstance(angle, (int, float, tuple)) or angle is None):
            raise TypeError(
                f"Invalid argument type. Expected float or str but got {type(angle)}"
            )
        if plane is None:
            plane = "XY"
        plane = plane.upper()
        if plane not in _PLANES:
            raise ValueError(f"Plane {plane} is not supported.")
        if plane == "XYZ":
            warnings.warn("Plane XYZ might be unstable. Use at your own risk.")
        if plane in ("X", "Y", "Z"):
            if angle is not None and angle != 0:
                raise ValueError(f"Plane {plane} does not support angle.")
            angle = 0
        self._plane = plane
        self._angle = angle
        self._node_id = -1

    def __repr__(self) -> str:
        if isinstance(self._angle, (int, float)):
            theta = round(self._angle, 4)
        elif isinstance(self._angle, tuple):
            theta = tuple(round(a, 4) for a in self._angle)
        else:
            theta = "θ"
        return f"Ment({theta}, {self._plane})"

    @property
    def plane(self) -> str:
        return self._plane

    @property
    def angle(self):
        return self._angle

    @property
    def node_id(self):
        return self._node_id

    @node_id.setter
    def node_id(self, value):
        self._node_id = value

    def set_angle(self, angle):
        self._angle = angle
        return self

    def copy(self) -> "Ment":
        return Ment(self._angle, self._plane)

    def is_trainable(self) -> bool:
        return self._angle is None and self._plane in ("XY", "XZ", "YZ", "XYZ")

    def matrix(self, angle=None, *args, **kwargs) -> np.ndarray:
        """The observable M whose +1 eigenprojector is outcome 0 (ment.py:218-253)."""
        if self._angle is None and angle is None:
            raise ValueError("Measurement is trainable, please provide an angle.")
        if self._angle is not None and angle is not None and self._angle != angle:
            raise ValueError(f"Measurement has a fixed angle of {round(self._angle, 4)}")
        if self._angle is not None:
            angle = self._angle
        p = self._plane
        if p == "XY":
            return np.cos(angle) * _PAULI_X + np.sin(angle) * _PAULI_Y
        if p == "X":
            return _PAULI_X.copy()
        if p == "Y":
            return _PAULI_Y.copy()
        if p == "Z":
            return _PAULI_Z.copy()
        if p == "XZ":
            return np.cos(angle) * _PAULI_X + np.sin(angle) * _PAULI_Z
        if p == "YZ":
            return np.cos(angle) * _PAULI_Y + np.sin(angle) * _PAULI_Z
        if not isinstance(angle, tuple):
            raise TypeError(f"Invalid argument type. Expected tuple but got {type(angle)}")
        a1, a2 = angle
        return (
            np.cos(a1) * np.cos(a2) * _PAULI_X
            + np.sin(a1) * np.cos(a2) * _PAULI_Y
            + np.sin(a2) * _PAULI_Z
        )

    def get_povm(self, angle=None, *args, **kwargs):
        """Projectors (I +/- M)/2 for outcomes 0 and 1 (ment.py:255-260)."""
        m = self.matrix(angle)
        eye = np.eye(2)
        return (eye + m) / 2, (eye - m) / 2


Measurement = Ment


class GraphState(nx.Graph):
    """Undirected graph of the resource state (a networkx graph)."""

    def __repr__(self) -> str:
        return f"GraphState with {self.number_of_nodes()} nodes and {self.number_of_edges()} edges."

    def __len__(self) -> int:
        return self.number_of_nodes()


# --------------------------------------------------------------------------
# causal flow
# --------------------------------------------------------------------------


def find_cflow(graph, input_nodes, output_nodes):
    """Causal flow of an open graph, or ``(None, None, None, None)``.

    The layer-by-layer search of Mhalla and Perdrix (arXiv:0709.2670), in the
    form mentpy runs it (mentpy/mbqc/flow.py:115-185): start from the outputs
    that have exactly one unprocessed neighbour, assign that neighbour as the
    flow predecessor, and peel layers until no candidate is left.  The candidate
    sets are Python sets iterated in their own order, as there, because the
    order decides which of two competing candidates wins a tie.

    Returns ``(flow, partial_order, depth, layers)``: ``flow(u)`` is the
    successor of ``u``, ``partial_order(u, v)`` is ``layer[u] > layer[v]``.
    """
    if len(input_nodes) != len(output_nodes):
        raise ValueError(
            f"Cannot find flow or gflow. Input ({len(input_nodes)}) and output "
            f"({len(output_nodes)}) nodes have different size."
        )
    layer = {v: 0 for v in graph.nodes()}
    past = {v: 0 for v in graph.nodes()}
    succ: Dict = {}
    outputs = set(output_nodes)
    inputs = set(input_nodes)
    non_outputs = set(graph.nodes() - set(output_nodes))

    frontier = set()
    for v in set(output_nodes) - set(input_nodes):
        past[v] = len(set(graph.neighbors(v)) & non_outputs)
        if past[v] == 1:
            frontier = frontier.union({v})

    all_nodes = set(graph.nodes())
    k = 1
    while True:
        nxt = set()
        for v in frontier:
            cand = set(graph.neighbors(v)) & (all_nodes - outputs)
            if len(cand) != 1:
                continue
            u = cand.pop()
            succ[u] = v
            layer[u] = k
            outputs.add(u)
            if u not in inputs:
                past[u] = len(set(graph.neighbors(u)) & (all_nodes - outputs))
                if past[u] == 1:
                    nxt.add(u)
            for w in set(graph.neighbors(u)):
                if past[w] > 0:
                    past[w] -= 1
                    if past[w] == 1:
                        nxt.add(w)
        if not nxt:
            break
        frontier = nxt
        k += 1

    if len(succ) != graph.number_of_nodes() - len(output_nodes):
        return None, None, None, None
    depth = max(succ.values()) if succ else 0
    return (lambda x: succ[x]), (lambda u, v: layer[u] > layer[v]), depth, layer


# --------------------------------------------------------------------------
# MBQCircuit
# --------------------------------------------------------------------------


class MBQCircuit:
    """An open graph with measurements: what one windowed sweep simulates.

    Keeps the attributes the windowed simulators read
    (mentpy/mbqc/mbqcircuit.py:56-158): ``graph``, ``input_nodes``,
    ``output_nodes``, ``measurements`` (insertion-ordered dict),
    ``trainable_nodes`` (measurement-dict order, the layout of the angle
    vector), ``quantum_output_nodes``, ``flow`` and ``measurement_order``.
    """

    def __init__(
        self,
        graph,
        input_nodes: List[int] = [],
        output_nodes: List[int] = [],
        measurements: Optional[dict] = None,
        default_measurement: Optional[Ment] = Ment("XY"),
        flow: Optional[Callable] = None,
        partial_order: Optional[Callable] = None,
        measurement_order: Optional[List[int]] = None,
        relabel_indices: bool = True,
    ) -> None:
        if relabel_indices:
            mapping = dict(zip(sorted(graph.nodes), range(graph.number_of_nodes())))
            inverse = {v: k for k, v in mapping.items()}
            graph = nx.relabel_nodes(graph, mapping)
            input_nodes = [mapping[i] for i in input_nodes]
            output_nodes = [mapping[i] for i in output_nodes]
            if flow is not None:
                user_flow = flow
                flow = lambda x: mapping[user_flow(inverse[x])]
            if partial_order is not None:
                user_po = partial_order
                partial_order = lambda x, y: user_po(inverse[x], inverse[y])
            if measurement_order is not None:
                measurement_order = [mapping[i] for i in measurement_order]
            if measurements is not None:
                measurements = {mapping[k]: v for k, v in measurements.items()}

        self._graph = graph
        missing_in = [v for v in input_nodes if v not in graph.nodes]
        if missing_in:
            raise ValueError(f"Input nodes {input_nodes} are not in the graph. Graph nodes are {graph.nodes}")
        if any(v not in graph.nodes for v in output_nodes):
            raise ValueError(f"Output nodes {output_nodes} are not in the graph. Graph nodes are {graph.nodes}")
        self._input_nodes = list(input_nodes)
        self._output_nodes = list(output_nodes)
        if not isinstance(default_measurement, Ment):
            raise ValueError(f"Default measurement {default_measurement} is not an instance of Ment.")
        self._default_measurement = default_measurement

        outputc = self.outputc
        if measurements is None:
            measurements = {node: default_measurement for node in outputc}
            for node in self._output_nodes:
                measurements[node] = None
        else:
            measurements = dict(measurements)
            bad = [v for v in measurements if v not in graph.nodes]
            if bad:
                raise ValueError(f"Nodes {bad} are not in the graph.")
            if not all(isinstance(v, Ment) or v is None for v in measurements.values()):
                raise ValueError(f"Values {measurements.values()} are not instances of Ment.")
            for node in graph.nodes:
                if node not in measurements:
                    measurements[node] = default_measurement if node in outputc else None
        self._measurements = measurements
        self._flow = None
        self._partial_order = None
        self._update_attributes()

        if flow is None or partial_order is None:
            flow, partial_order, _depth, _layers = find_cflow(graph, self._input_nodes, self._output_nodes)
        self._flow = flow
        self._partial_order = partial_order

        if measurement_order is None and flow is not None:
            measurement_order = self.calculate_order()
        self._quantum_output_nodes = [n for n, m in self._measurements.items() if m is None]
        self._measurement_order = measurement_order

    # ---------------------------------------------------------------- access
    def __repr__(self) -> str:
        return f"MBQCircuit with {self._graph.number_of_nodes()} qubits."

    def __len__(self) -> int:
        return self._graph.number_of_nodes()

    def __getitem__(self, key):
        try:
            return self._measurements[key]
        except KeyError:
            raise ValueError(f"Node {key} is not in the graph.")

    def __setitem__(self, key, value):
        if key not in self._graph.nodes:
            raise ValueError(f"Node {key} is not in the graph.")
        if not isinstance(value, Ment):
            raise ValueError(f"Value {value} is not a Measurement object.")
        self._measurements[key] = value
        self._update_attributes()

    @property
    def graph(self):
        return self._graph

    @property
    def input_nodes(self) -> List[int]:
        return self._input_nodes

    @property
    def output_nodes(self) -> List[int]:
        return self._output_nodes

    @property
    def measurements(self) -> dict:
        return self._measurements

    @property
    def quantum_output_nodes(self) -> List[int]:
        return self._quantum_output_nodes

    @property
    def trainable_nodes(self) -> List[int]:
        return self._trainable_nodes

    @trainable_nodes.setter
    def trainable_nodes(self, nodes: List[int]) -> None:
        if not all(v in self._graph.nodes for v in nodes):
            raise ValueError(f"Trainable nodes {nodes} are not in the graph.")
        self._trainable_nodes = list(nodes)

    @property
    def flow(self):
        return self._flow

    @property
    def partial_order(self):
        return self._partial_order

    @property
    def measurement_order(self) -> Optional[List[int]]:
        return self._measurement_order

    @property
    def outputc(self) -> List[int]:
        return [v for v in self._graph.nodes() if v not in self._output_nodes]

    @property
    def inputc(self) -> List[int]:
        return [v for v in self._graph.nodes() if v not in self._input_nodes]

    # -------------------------------------------------------------- internals
    def _update_attributes(self) -> None:
        """Trainable nodes and quantum outputs in measurement-dict order
        (mbqcircuit.py:325-353)."""
        trainable, quantum_out = [], []
        for node, ment in self._measurements.items():
            if ment is not None:
                if ment.is_trainable():
                    trainable.append(node)
                ment = copy.deepcopy(ment)
                ment.node_id = node
                self._measurements[node] = ment
            elif node in self._output_nodes:
                quantum_out.append(node)
        self._trainable_nodes = trainable
        self._quantum_output_nodes = quantum_out

    def calculate_order(self) -> List[int]:
        """Measurement order: nodes sorted by how many nodes they precede
        (descending; ties in graph node order), inputs moved to the front in
        input order (mbqcircuit.py:390-422)."""
        nodes = list(self._graph.nodes())
        po = self._partial_order
        counts = [sum(1 for j in nodes if po(i, j)) for i in nodes]
        groups: Dict[int, List[int]] = {}
        for idx, c in enumerate(counts):
            groups.setdefault(c, []).append(nodes[idx])
        order = [n for c in sorted(groups, reverse=True) for n in groups[c]]
        for i in self._input_nodes[::-1]:
            order.remove(i)
            order.insert(0, i)
        return order

    def add_edge(self, u, v) -> None:
        """Add an edge and rebuild the circuit with default measurements
        (mbqcircuit.py:424-432)."""
        self._graph.add_edge(u, v)
        try:
            self.__init__(self._graph, self._input_nodes, self._output_nodes)
        except Exception as exc:  # keep the graph unchanged on failure
            self._graph.remove_edge(u, v)
            raise ValueError(f"Cannot add edge between {u} and {v}.\n{exc}")


# --------------------------------------------------------------------------
# stacking and templates
# --------------------------------------------------------------------------


def _hstack2(a: MBQCircuit, b: MBQCircuit) -> MBQCircuit:
    """Glue the outputs of ``a`` onto the inputs of ``b`` (mbqcircuit.py:561-611)."""
    if len(a.output_nodes) != len(b.input_nodes):
        raise ValueError(
            "The output of the first state must be the same size as the input of the second state."
        )
    graph = nx.disjoint_union(a.graph, b.graph)
    na = list(a.graph.nodes())
    nb = list(b.graph.nodes())
    shift = len(na)
    for i in range(len(a.output_nodes)):
        graph.add_edge(na.index(a.output_nodes[i]), nb.index(b.input_nodes[i]) + shift)
    inputs = [na.index(i) for i in a.input_nodes]
    outputs = [nb.index(j) + shift for j in b.output_nodes]
    meas = {na.index(i): m for i, m in a.measurements.items()}
    meas.update({nb.index(i) + shift: m for i, m in b.measurements.items()})
    n_a = a.graph.number_of_nodes()
    for i, j in zip(a.output_nodes, b.input_nodes):
        graph.add_edge(i, j + n_a)
        graph = nx.contracted_edge(graph, (j + n_a, i), self_loops=False)
        del meas[i]
    return MBQCircuit(graph, inputs, outputs, measurements=meas)


def hstack(circuits) -> MBQCircuit:
    """Concatenate circuits along their wires."""
    circuits = list(circuits)
    if not circuits:
        raise ValueError("Cannot horizontally stack an empty list of states.")
    return reduce(_hstack2, circuits)


def linear_cluster(n: int, **kwargs) -> MBQCircuit:
    """1D cluster of ``n`` qubits, input 0, output n-1 (templates.py:16-45)."""
    g = GraphState()
    g.add_edges_from([(i, i + 1) for i in range(n - 1)])
    return MBQCircuit(g, input_nodes=[0], output_nodes=[n - 1], **kwargs)


def many_wires(n_wires: List[int], **kwargs) -> MBQCircuit:
    """Disconnected 1D wires of the given lengths (templates.py:48-91)."""
    if not all(isinstance(n, int) and n > 1 for n in n_wires):
        raise ValueError("n_wires must be a list of integers greater than 1")
    g = GraphState()
    starts = [sum(n_wires[:i]) for i in range(len(n_wires))]
    for s, n in zip(starts, n_wires):
        g.add_edges_from([(s + j, s + j + 1) for j in range(n - 1)])
    ends = [s + n - 1 for s, n in zip(starts, n_wires)]
    return MBQCircuit(g, input_nodes=starts, output_nodes=ends, **kwargs)


def grid_cluster(n: int, m: int, periodic: bool = False, **kwargs) -> MBQCircuit:
    """``n`` rows of ``m`` qubits with vertical links (templates.py:94-147)."""
    g = GraphState()
    for r in range(n):
        g.add_edges_from([(r * m + j, r * m + j + 1) for j in range(m - 1)])
    for r in range(n - 1):
        g.add_edges_from([(r * m + j, (r + 1) * m + j) for j in range(m)])
    if periodic and n > 1:
        for j in range(m):
            g.add_edge(j, (n - 1) * m + j)
    return MBQCircuit(
        g,
        input_nodes=[r * m for r in range(n)],
        output_nodes=[r * m + m - 1 for r in range(n)],
        **kwargs,
    )


def muta(n_wires: int, n_layers: int, **kwargs) -> MBQCircuit:
    """Multiple Triangle Ansatz (templates.py:150-216): per wire, a block of
    ``n_wires`` 5-qubit wires whose second qubit is linked to the first and
    third qubit of every other wire; blocks and layers glued by ``hstack``."""
    options = {"restrict_trainable": True, "one_column": False}
    options.update(kwargs)
    size = 5
    block = None
    for wire in range(n_wires):
        if options["one_column"] and wire != 0:
            break
        g = many_wires([size] * n_wires)
        if options["restrict_trainable"]:
            # only survives when no edge is added below (a single wire); an
            # added edge rebuilds the circuit, as in the reference
            g.trainable_nodes = list(
                set(g.trainable_nodes) - set([i - 1 for i in g.output_nodes])
            )
        for other in range(n_wires):
            if other != wire:
                g.add_edge(size * wire + 1, size * other)
                g.add_edge(size * wire + 1, size * other + 2)
        block = g if block is None else hstack((block, g))
    out = None
    for _ in range(n_layers):
        out = block if out is None else hstack((out, block))
    return out
