"""Window-plan compiler: MBQCircuit -> flat per-step tables for the kernels.

The windowed sweep of mentpy's numpy simulators keeps a window of ``w`` qubits
(the next ``w`` nodes of the schedule).  At step ``k`` it measures window slot
0 (node ``schedule[k]``), traces it out, appends node ``schedule[k+w]`` in
``|+>`` and applies a CZ between it and each graph neighbour still in the window
(mentpy/simulators/np_simulator_sv.py:164-225, np_simulator_dm.py:151-216).

The GPU kernels run the same sweep *in place*: every window slot is a fixed
physical bit of the amplitude index, and the qubit that enters at step ``k``
takes the bit that the measured qubit frees.  With the initial window laid out
as ``schedule[j] -> bit j`` this makes the bit measured at step ``k`` simply
``k mod w``, and each step a single pass over the window.  This module turns a
circuit into the tables that describe that pass:

* ``in_bits[i]``    -- physical bit of input qubit ``i`` (input_nodes order),
* ``init_cz[q]``    -- CZ partners (bit mask, higher bits only) of bit ``q``
                       inside the first window,
* ``step_mask[k]``  -- CZ partners of the qubit entering at step ``k``, or
                       ``DEAD`` when no qubit enters (the window shrinks),
* ``step_angle[k]`` -- index into the angle vector, or -1 for a fixed angle,
* ``step_plane[k]`` / ``step_fixed_angle[k]`` -- the measurement basis,
* ``out_bits[j]``   -- physical bit of output qubit ``j`` in the order the
                       reference returns them.

The bookkeeping follows the reference exactly: schedule and window choice
(np_simulator_sv.py:61-100, np_simulator_dm.py:47-85), the input reorder
(np_simulator_sv.py:81-86), the angle lookup through ``trainable_nodes``
(np_simulator_sv.py:245-252), and the output reorder rules
(np_simulator_sv.py:286-290, np_simulator_dm.py:267-273).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

__all__ = ["WindowPlan", "compile_plan", "DEAD", "PLANE_CODES"]

DEAD = 1 << 31
PLANE_CODES = {"XY": 0, "X": 1, "Y": 2, "XZ": 3, "YZ": 4, "Z": 5}
MAX_WINDOW = 30


@dataclass
class WindowPlan:
    kind: str                     # "sv" or "dm"
    window: int                   # w
    n_nodes: int                  # N = nodes in the graph
    schedule: List[int]           # full measurement order
    schedule_measure: List[int]   # nodes measured by the sweep, in order
    n_in: int
    n_out: int
    n_angles: int                 # len(trainable_nodes)
    trainable_nodes: List[int]
    in_bits: np.ndarray           # int32 [n_in]
    init_cz: np.ndarray           # uint32 [w]
    step_mask: np.ndarray         # uint32 [M]
    step_angle: np.ndarray        # int32 [M]
    step_plane: np.ndarray        # int32 [M]
    step_fixed_angle: np.ndarray  # float64 [M]
    out_bits: np.ndarray          # int32 [n_out]
    out_nodes: List[int]          # output labels in returned order
    output_ment_nodes: List[int] = field(default_factory=list)  # SV: outputs carrying a Ment

    @property
    def n_steps(self) -> int:
        return len(self.schedule_measure)

    def outcome_nodes(self) -> List[int]:
        return list(self.schedule_measure) + list(self.output_ment_nodes)


def _find_swaps(source, target):
    """Transpositions turning ``source`` into ``target`` (np_simulator_sv.py:360-374)."""
    assert set(source) == set(target), (
        f"Both lists must have the same elements, but source={source} and target={target}"
    )
    src = list(source)
    swaps = []
    for i, t in enumerate(target):
        if src[i] != t:
            j = src.index(t, i + 1)
            src[i], src[j] = src[j], src[i]
            swaps.append((i, j))
    return swaps


def _permuted(labels, target):
    """Labels after applying the reference's swap sequence; asserts like it."""
    _find_swaps(labels, target)
    return list(target)


def _neighbors(graph, node):
    return list(graph.neighbors(node))


def compile_plan(
    circuit,
    kind: str = "sv",
    window_size: int = 1,
    schedule: Optional[List[int]] = None,
    force0: bool = True,
    dev_mode: bool = False,
    extended_planes: bool = False,
) -> WindowPlan:
    """Compile ``circuit`` into a window plan for the ``sv`` or ``dm`` sweep.

    Raises the same exceptions, for the same inputs, as the constructors of
    ``NumpySimulatorSV``/``NumpySimulatorDM`` (np_simulator_sv.py:38-128,
    np_simulator_dm.py:33-115).  ``extended_planes=True`` lets a statevector
    plan measure in the XZ and YZ planes too (the reference statevector
    simulator rejects them, np_simulator_sv.py:53-59; its density-matrix
    simulator takes them, and the statevector kernels then apply the
    reference's own step to them).
    """
    if kind not in ("sv", "dm"):
        raise ValueError(f"unknown sweep kind {kind!r}")
    if not force0:
        raise NotImplementedError("Numpy simulator does not support force0=False.")
    if dev_mode:
        raise NotImplementedError("dev_mode wire scheduling is not supported by the GPU backend.")

    graph = circuit.graph
    output_nodes = list(circuit.output_nodes)
    input_nodes = list(circuit.input_nodes)
    qout = list(circuit.quantum_output_nodes)

    if kind == "sv":
        for node in graph.nodes:
            m = circuit[node]
            allowed = ("X", "Y", "XY", "XZ", "YZ") if extended_planes else ("X", "Y", "XY")
            if m is not None and m.plane not in allowed:
                raise ValueError(
                    f"Node {node} has plane {m.plane}, but only XY plane is supported."
                )

    excluded = output_nodes if kind == "sv" else qout
    w = window_size
    if schedule is not None:
        schedule = list(schedule)
        sched_meas = [i for i in schedule if i not in excluded]
    elif circuit.measurement_order is not None:
        schedule = list(circuit.measurement_order)
        sched_meas = [i for i in schedule if i not in excluded]
        if w == 1 and circuit.flow is not None:
            w = len(input_nodes) + 1
    else:
        raise ValueError(
            "Schedule must be provided for numpy simulator as the MBQCircuit does not have a flow."
        )

    n_in = len(input_nodes)
    # input reorder: kron position t <- qubit schedule[t] (np_simulator_sv.py:81-86)
    _find_swaps(input_nodes, schedule[:n_in])
    if n_in > w:
        raise ValueError(
            f"Input state has {n_in} qubits, but window size is set to {w}."
            " Input state must have at most as many qubits as the window size minus one."
        )
    if w > len(sched_meas):
        raise ValueError(
            f"Window size is set to {w}, but schedule only has {len(sched_meas)} measurements."
        )
    if w > MAX_WINDOW:
        raise ValueError(f"window size {w} exceeds the supported maximum of {MAX_WINDOW}")
    if len(schedule) < w:
        raise ValueError("schedule is shorter than the window")

    N = graph.number_of_nodes()
    M = len(sched_meas)
    bit_of_pos = lambda pos: pos % w  # noqa: E731 -- slot of schedule position

    pos_of = {}
    for t, node in enumerate(schedule):
        pos_of.setdefault(node, t)
    in_bits = np.array([bit_of_pos(schedule.index(n)) for n in input_nodes], dtype=np.int32)

    # initial CZ layer inside the first window (np_simulator_sv.py:107-128)
    window0 = schedule[:w]
    init_cz = np.zeros(w, dtype=np.uint32)
    wset = set(window0)
    for t, node in enumerate(window0):
        for nb in _neighbors(graph, node):
            if nb in wset:
                tb = window0.index(nb)
                if tb > t:
                    init_cz[t] |= np.uint32(1 << tb)

    trainable = list(circuit.trainable_nodes)
    step_mask = np.zeros(M, dtype=np.uint32)
    step_angle = np.full(M, -1, dtype=np.int32)
    step_plane = np.zeros(M, dtype=np.int32)
    step_fixed = np.zeros(M, dtype=np.float64)
    for k in range(M):
        node = sched_meas[k]
        ment = circuit[node]
        if ment is None:
            raise ValueError(f"Node {node} is scheduled for measurement but carries no Ment.")
        plane = ment.plane
        if plane not in PLANE_CODES:
            raise NotImplementedError(
                f"Plane {plane} is not supported by the GPU {kind} sweep (node {node})."
            )
        step_plane[k] = PLANE_CODES[plane]
        if node in trainable:
            step_angle[k] = trainable.index(node)
        else:
            step_fixed[k] = float(ment.angle)
        # qubit entering after step k (np_simulator_sv.py:207-223)
        if k + 1 + w <= N:
            if k + w >= len(schedule):
                raise ValueError("schedule does not cover the window at step %d" % k)
            new = schedule[k + w]
            win = schedule[k + 1 : k + 1 + w]
            mask = 0
            for nb in _neighbors(graph, new):
                if nb in win and nb != new:
                    mask |= 1 << bit_of_pos(k + 1 + win.index(nb))
            step_mask[k] = mask
        else:
            step_mask[k] = DEAD

    # qubits left in the window after the sweep, in kron order
    remaining = list(schedule[M : M + w])
    n_left = min(w, N - M)
    if len(remaining) != n_left:
        raise ValueError("schedule does not cover the final window")
    output_ment_nodes: List[int] = []
    if kind == "sv":
        for i in output_nodes:
            m = circuit[i]
            if m is not None:
                if m.angle is None:
                    raise ValueError("Measurement is trainable, please provide an angle.")
                if i < n_left:
                    raise NotImplementedError(
                        "measured output node whose label is below the final window size"
                    )
                output_ment_nodes.append(i)
        current = remaining
        final = list(output_nodes) if qout != current else current
        if final != current:
            final = _permuted(current, final)
        labels_at = current
    else:
        current = [i for i in schedule if i not in sched_meas]
        if len(current) != n_left:
            raise ValueError("remaining window does not match the quantum outputs")
        final = list(qout) if qout != current else current
        if final != current:
            final = _permuted(current, final)
        labels_at = current
    out_bits = np.array(
        [bit_of_pos(M + labels_at.index(lbl)) for lbl in final], dtype=np.int32
    )

    return WindowPlan(
        kind=kind,
        window=w,
        n_nodes=N,
        schedule=schedule,
        schedule_measure=sched_meas,
        n_in=n_in,
        n_out=len(final),
        n_angles=len(trainable),
        trainable_nodes=trainable,
        in_bits=in_bits,
        init_cz=init_cz,
        step_mask=step_mask,
        step_angle=step_angle,
        step_plane=step_plane,
        step_fixed_angle=step_fixed,
        out_bits=out_bits,
        out_nodes=final,
        output_ment_nodes=output_ment_nodes,
    )
