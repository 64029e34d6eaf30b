"""complex128 restatement of mentpy's windowed sweep, O(2^w) per step.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__``).

The bookkeeping is restated directly from the reference simulators, with the
window kept as a list of node labels exactly as they keep it, so that this
module shares no code with the GPU plan compiler it checks:

* schedule / window selection  -- np_simulator_sv.py:61-100, np_simulator_dm.py:47-85
* input reorder and padding    -- np_simulator_sv.py:81-86,103-104
* initial CZ layer             -- np_simulator_sv.py:107-128, np_simulator_dm.py:93-114
* measurement of slot 0        -- np_simulator_sv.py:164-225,322-358 (force0: outcome 0)
                                  np_simulator_dm.py:151-216,307-346 (outcome 1 iff prob0 < 1e-4)
* projectors (I +/- M)/2       -- ment.py:218-260
* partial traces               -- state_ops.py:42-74 (sum over the index, then renormalise)
                                  state_ops.py:77-119 (proper trace)
* output reorder               -- np_simulator_sv.py:278-297, np_simulator_dm.py:267-283

Only the linear algebra differs: operators act on one tensor axis instead of
being expanded by ``kron`` to 2^w x 2^w matrices.

Depolarising noise (``noise_p``) is an extension, absent from the reference
numpy path: each qubit passes once through the single-qubit depolarising
channel, right before it is measured (output qubits: after the sweep).  That is
PennyLane's placement (pennylane_simulator.py:123-126: every wire once, after
the CZ layer) seen through the window.
"""
from __future__ import annotations

import numpy as np

_X = np.array([[0, 1], [1, 0]], dtype=complex)
_Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
_Z = np.array([[1, 0], [0, -1]], dtype=complex)
_PLUS = np.array([1, 1], dtype=complex) / np.sqrt(2)


def observable(plane: str, angle) -> np.ndarray:
    """Ment.matrix (ment.py:218-253)."""
    if plane == "XY":
        return np.cos(angle) * _X + np.sin(angle) * _Y
    if plane == "X":
        return _X
    if plane == "Y":
        return _Y
    if plane == "Z":
        return _Z
    if plane == "XZ":
        return np.cos(angle) * _X + np.sin(angle) * _Z
    if plane == "YZ":
        return np.cos(angle) * _Y + np.sin(angle) * _Z
    raise ValueError(f"plane {plane}")


def povm(plane: str, angle):
    m = observable(plane, angle)
    return (np.eye(2) + m) / 2, (np.eye(2) - m) / 2


def schedule_for(circuit, kind: str, window_size: int = 1, schedule=None):
    """(schedule, schedule_measure, w) as the reference constructors pick them."""
    excl = circuit.output_nodes if kind == "sv" else circuit.quantum_output_nodes
    w = window_size
    if schedule is not None:
        sched = list(schedule)
    elif circuit.measurement_order is not None:
        sched = list(circuit.measurement_order)
        if w == 1 and circuit.flow is not None:
            w = len(circuit.input_nodes) + 1
    else:
        raise ValueError("Schedule must be provided for numpy simulator as the MBQCircuit does not have a flow.")
    meas = [i for i in sched if i not in excl]
    n_in = len(circuit.input_nodes)
    if n_in > w:
        raise ValueError("Input state has more qubits than the window size.")
    if w > len(meas):
        raise ValueError("Window size larger than the number of measurements.")
    return sched, meas, w


def _perm_state(vec, cur, target):
    """Vector with qubit label order ``cur`` rewritten in order ``target``."""
    n = len(cur)
    assert set(cur) == set(target)
    t = vec.reshape([2] * n)
    t = np.transpose(t, [cur.index(x) for x in target])
    return t.reshape(-1)


def _perm_rho(rho, cur, target):
    n = len(cur)
    assert set(cur) == set(target)
    p = [cur.index(x) for x in target]
    t = rho.reshape([2] * (2 * n))
    t = np.transpose(t, p + [n + i for i in p])
    return t.reshape(2**n, 2**n)


def _op_on(vec, op, slot, n):
    t = vec.reshape(2**slot, 2, 2 ** (n - slot - 1))
    return np.einsum("ab,ibj->iaj", op, t).reshape(-1)


def _op_on_rho(rho, op, slot, n):
    d = 2**n
    t = rho.reshape(2**slot, 2, 2 ** (n - slot - 1), d)
    t = np.einsum("ab,ibjk->iajk", op, t).reshape(d, d)
    t = t.reshape(d, 2**slot, 2, 2 ** (n - slot - 1))
    t = np.einsum("kibj,ab->kiaj", t, op.conj()).reshape(d, d)
    return t


def _cz_sign(n, a, b):
    idx = np.arange(2**n)
    ba = (idx >> (n - 1 - a)) & 1
    bb = (idx >> (n - 1 - b)) & 1
    return np.where(ba & bb, -1.0, 1.0)


def _depolarise_slot(rho, slot, n, p):
    if p == 0.0:
        return rho
    d = 2**n
    out = (1 - p) * rho
    for P in (_X, _Y, _Z):
        out = out + (p / 3) * _op_on_rho(rho, P, slot, n)
    return out


def _angle_for(circuit, node, angles):
    trainable = list(circuit.trainable_nodes)
    if node in trainable:
        return angles[trainable.index(node)]
    return circuit[node].angle


def _initial(circuit, sched, w, input_state):
    n_in = len(circuit.input_nodes)
    if input_state is None:
        input_state = np.ones(2**n_in, dtype=complex) / np.sqrt(2**n_in)
    vec = _perm_state(np.asarray(input_state, dtype=complex), list(circuit.input_nodes), sched[:n_in])
    for _ in range(w - n_in):
        vec = np.kron(vec, _PLUS)
    win = sched[:w]
    g = circuit.graph
    for a, na in enumerate(win):
        for nb in g.neighbors(na):
            if nb in win and na < nb:
                vec = vec * _cz_sign(w, a, win.index(nb))
    return vec


def run_sv(circuit, angles, input_state=None, window_size=1, schedule=None, output_form="dm"):
    """Forward sweep of ``NumpySimulatorSV`` (np_simulator_sv.py:227-297).

    Returns ``(state, outcomes, probs)`` where ``probs[k]`` is prob0 of step k.
    """
    sched, meas, w = schedule_for(circuit, "sv", window_size, schedule)
    angles = np.asarray(angles, dtype=float)
    if len(angles) != len(circuit.trainable_nodes):
        raise ValueError("Number of angles does not match number of trainable nodes.")
    N = circuit.graph.number_of_nodes()
    psi = _initial(circuit, sched, w, input_state)
    outcomes, probs = {}, []
    g = circuit.graph
    for k, node in enumerate(meas):
        ment = circuit[node]
        n_cur = min(w, N - k)
        p0, _ = povm(ment.plane, _angle_for(circuit, node, angles))
        proj = _op_on(psi, p0, 0, n_cur)
        probs.append(float(np.real(np.vdot(psi, proj))))
        with np.errstate(invalid="ignore", divide="ignore"):
            psi = proj / np.linalg.norm(proj)
            psi = psi.reshape(2, -1).sum(axis=0)
            psi = psi / np.linalg.norm(psi)
        outcomes[node] = 0
        if k + 1 + w <= N:
            psi = np.kron(psi, _PLUS)
            win = sched[k + 1 : k + 1 + w]
            new = win[-1]
            for nb in g.neighbors(new):
                if nb in win:
                    psi = psi * _cz_sign(w, win.index(nb), w - 1)
    M = len(meas)
    n_cur = min(w, N - M)
    for i in circuit.output_nodes:
        ment = circuit[i]
        if ment is not None:
            p0, _ = povm(ment.plane, ment.angle)
            if i < n_cur:
                psi = _op_on(psi, p0, i, n_cur)
                psi = psi / np.linalg.norm(psi)
            outcomes[i] = 0
    current = sched[M : M + w]
    if list(circuit.quantum_output_nodes) != current:
        psi = _perm_state(psi, current, list(circuit.output_nodes))
    if output_form.lower() in ("dm", "densitymatrix"):
        return np.outer(psi, psi.conj()), outcomes, probs
    if output_form.lower() in ("sv", "statevector"):
        return psi, outcomes, probs
    raise ValueError(f"Output form {output_form} is not supported.")


def _eigvec(plane: str, angle, outcome: int):
    """Unit eigenvector of Ment.matrix with eigenvalue +1 (outcome 0) or -1
    (outcome 1): the range of the projector povm(plane, angle)[outcome]."""
    p = povm(plane, angle)[outcome]
    j = int(np.argmax(np.linalg.norm(p, axis=0)))
    v = p[:, j]
    return v / np.linalg.norm(v)


def run_sv_sampled(circuit, angles, input_state, outcomes, window_size=1, schedule=None):
    """The PennyLane backend's sampled circuit (pennylane_simulator.py:114-153:
    each non-output node measured, on outcome 1 an X on flow(node) and a Z on
    every neighbour of flow(node) measured after node) swept through the
    reference's statevector window (np_simulator_sv.py:227-297), with the
    drawn ``outcomes[node]`` given.  The corrections act as gates: at once on
    nodes in the window, and for a Z on a node not yet added, when it is added
    (Z commutes with the CZ layer).  An X on a window node f comes before the
    CZs of f with nodes not yet added, where the whole circuit has it after
    them: X_f CZ_fn = CZ_fn X_f Z_n, so each such n also gets a Z on arrival.
    The measured node is projected onto the
    eigenvector of its outcome and contracted out.  Returns the normalised
    amplitudes over ``circuit.output_nodes`` (global phase arbitrary)."""
    sched, meas, w = schedule_for(circuit, "sv", window_size, schedule)
    angles = np.asarray(angles, dtype=float)
    N = circuit.graph.number_of_nodes()
    g = circuit.graph
    mo = list(circuit.measurement_order)
    pos = {v: i for i, v in enumerate(mo)}
    psi = _initial(circuit, sched, w, input_state)
    win = list(sched[:w])
    added = set(win)
    pending_z = set()
    for k, node in enumerate(meas):
        assert win[0] == node
        n_cur = len(win)
        ment = circuit[node]
        e = _eigvec(ment.plane, _angle_for(circuit, node, angles), int(outcomes[node]))
        psi = e.conj() @ psi.reshape(2, -1)
        psi = psi / np.linalg.norm(psi)
        win = win[1:]
        n_cur -= 1
        if int(outcomes[node]):
            f = circuit.flow(node)
            if f not in win:
                raise ValueError(f"flow({node}) = {f} is not in the window")
            psi = _op_on(psi, _X, win.index(f), n_cur)
            pending_z ^= {nb for nb in g.neighbors(f) if nb not in added}
            for nb in g.neighbors(f):
                if nb == node or pos.get(nb, N) <= pos[node]:
                    continue
                if nb in win:
                    psi = _op_on(psi, _Z, win.index(nb), n_cur)
                else:
                    pending_z ^= {nb}
        if k + 1 + w <= N:
            psi = np.kron(psi, _PLUS)
            new = sched[k + w]
            win.append(new)
            added.add(new)
            for nb in g.neighbors(new):
                if nb in win[:-1]:
                    psi = psi * _cz_sign(w, win.index(nb), w - 1)
            if new in pending_z:
                psi = _op_on(psi, _Z, w - 1, w)
                pending_z.discard(new)
    assert not pending_z, pending_z
    if win != list(circuit.output_nodes):
        psi = _perm_state(psi, win, list(circuit.output_nodes))
    return psi


def run_dm(circuit, angles, input_state=None, window_size=1, schedule=None, noise_p=0.0, mode="sample",
           z_outcomes=None):
    """Forward sweep of ``NumpySimulatorDM`` (np_simulator_dm.py:218-283).

    Returns ``(rho, outcomes, probs)``; raises ``ValueError`` on NaN like the
    reference (np_simulator_dm.py:179-182).  Z-basis steps follow
    ``measure_ment`` (np_simulator_dm.py:327-344): in ``mode="expectation"``
    the qubit is traced out unprojected and the outcome is prob1 / (prob0 +
    prob1); otherwise the outcome is drawn -- here taken from ``z_outcomes``
    (node -> 0/1), else from numpy's global generator as the reference does.
    """
    sched, meas, w = schedule_for(circuit, "dm", window_size, schedule)
    angles = np.asarray(angles, dtype=float)
    if len(angles) != len(circuit.trainable_nodes):
        raise ValueError("Number of angles does not match number of trainable nodes.")
    N = circuit.graph.number_of_nodes()
    psi = _initial(circuit, sched, w, input_state)
    rho = np.outer(psi, psi.conj())
    g = circuit.graph
    plus_dm = np.outer(_PLUS, _PLUS.conj())
    outcomes, probs = {}, []
    for k, node in enumerate(meas):
        ment = circuit[node]
        n_cur = min(w, N - k)
        rho = _depolarise_slot(rho, 0, n_cur, noise_p)
        p0, p1 = povm(ment.plane, _angle_for(circuit, node, angles))
        p0e = np.kron(p0, np.eye(2 ** (n_cur - 1)))
        p1e = np.kron(p1, np.eye(2 ** (n_cur - 1)))
        prob0 = float(np.real(np.trace(rho @ p0e)))
        prob1 = float(np.real(np.trace(rho @ p1e)))
        probs.append(prob0)
        expect = ment.plane == "Z" and mode in ("expectation", "exp")
        if expect:
            outcome = prob1 / (prob0 + prob1)
        elif ment.plane == "Z":
            if z_outcomes is not None:
                outcome = int(z_outcomes[node])
            else:
                outcome = int(np.random.choice([0, 1], p=np.array([prob0, prob1]) / (prob0 + prob1)))
        else:
            outcome = 1 if prob0 < 1e-4 else 0
        with np.errstate(invalid="ignore", divide="ignore"):
            if expect:
                pass  # no projection
            elif outcome == 0:
                rho = p0e @ rho @ p0e.conj().T / prob0
            else:
                rho = p1e @ rho @ p1e.conj().T / prob1
        if np.isnan(rho).any():
            raise ValueError("qstate has nan, you might want to increase the window size")
        outcomes[node] = outcome
        d = 2 ** (n_cur - 1)
        rho = rho.reshape(2, d, 2, d)
        rho = rho[0, :, 0, :] + rho[1, :, 1, :]
        if k + 1 + w <= N:
            rho = np.kron(rho, plus_dm)
            win = sched[k + 1 : k + 1 + w]
            new = win[-1]
            for nb in g.neighbors(new):
                if nb in win:
                    s = _cz_sign(w, win.index(nb), w - 1)
                    rho = rho * np.outer(s, s)
    M = len(meas)
    n_cur = min(w, N - M)
    for slot in range(n_cur):
        rho = _depolarise_slot(rho, slot, n_cur, noise_p)
    current = [i for i in sched if i not in meas]
    if list(circuit.quantum_output_nodes) != current:
        rho = _perm_rho(rho, current, list(circuit.quantum_output_nodes))
    return rho, outcomes, probs


def fidelity_pure(target, state):
    """|<t|z>|^2 for a pure target and a state vector or density matrix.
    Restates the fidelity the reference borrows from PennyLane
    (calculator/borrows.py:4-6) for a pure target."""
    target = np.asarray(target)
    state = np.asarray(state)
    if state.ndim == 1:
        return float(abs(np.vdot(target, state)) ** 2)
    return float(np.real(np.vdot(target, state @ target)))


# ---------------------------------------------------------------- batched
# The same sweeps vectorised over many runs of one circuit (leading batch
# axis), so that whole benchmark batches can be checked in seconds.  Same
# bookkeeping as ``run_sv`` / ``run_dm`` above, step for step.

def _povm_batch(plane: str, thetas):
    """(P0, P1) of shape [B, 2, 2] for per-run angles (ment.py:218-260)."""
    th = np.asarray(thetas, dtype=float)
    B = th.shape[0]
    obs = np.empty((B, 2, 2), dtype=complex)
    if plane in ("X", "Y", "Z"):
        obs[:] = observable(plane, 0.0)
    else:
        a, b = {"XY": (_X, _Y), "XZ": (_X, _Z), "YZ": (_Y, _Z)}[plane]
        obs[:] = np.cos(th)[:, None, None] * a + np.sin(th)[:, None, None] * b
    eye = np.eye(2)[None]
    return (eye + obs) / 2, (eye - obs) / 2


def _re_dot(a, b):
    """Re <a_r|b_r> for every row r."""
    return np.einsum("bi,bi->b", a.real, b.real) + np.einsum("bi,bi->b", a.imag, b.imag)


def _op_on_batch(vec, ops, slot, n):
    B = vec.shape[0]
    t = vec.reshape(B, 2**slot, 2, 2 ** (n - slot - 1))
    a0, a1 = t[:, :, 0, :], t[:, :, 1, :]
    o = ops.reshape(B, 2, 2, 1, 1)
    out = np.empty_like(t)
    out[:, :, 0, :] = o[:, 0, 0] * a0 + o[:, 0, 1] * a1
    out[:, :, 1, :] = o[:, 1, 0] * a0 + o[:, 1, 1] * a1
    return out.reshape(B, -1)


def _perm_state_batch(vec, cur, target):
    n = len(cur)
    B = vec.shape[0]
    t = vec.reshape([B] + [2] * n)
    t = np.transpose(t, [0] + [1 + cur.index(x) for x in target])
    return t.reshape(B, -1)


def _perm_rho_batch(rho, cur, target):
    n = len(cur)
    B = rho.shape[0]
    p = [cur.index(x) for x in target]
    t = rho.reshape([B] + [2] * (2 * n))
    t = np.transpose(t, [0] + [1 + i for i in p] + [1 + n + i for i in p])
    return t.reshape(B, 2**n, 2**n)


def _sandwich_batch(rho, ops, slot, n):
    """(op on ``slot``) rho (op on ``slot``)^dagger for every row: ``ops`` is
    one [2, 2] operator or one per row [B, 2, 2].  The slot's (row, column)
    bit pair is moved to the front and mixed by kron(op, conj(op)), a 4 x 4
    matrix per row."""
    B, d = rho.shape[0], 2**n
    hi, lo = 2**slot, 2 ** (n - slot - 1)
    t = rho.reshape(B, hi, 2, lo, hi, 2, lo).transpose(0, 2, 5, 1, 3, 4, 6).reshape(B, 4, -1)
    ops = np.broadcast_to(np.asarray(ops, dtype=complex), (B, 2, 2))
    k4 = np.einsum("bxa,byc->bxyac", ops, ops.conj()).reshape(B, 4, 4)
    out = np.matmul(k4, t).reshape(B, 2, 2, hi, lo, hi, lo)
    return out.transpose(0, 3, 1, 4, 5, 2, 6).reshape(B, d, d)


def _depolarise_slot_batch(rho, slot, n, p):
    if p == 0.0:
        return rho
    out = (1 - p) * rho
    for P in (_X, _Y, _Z):
        out = out + (p / 3) * _sandwich_batch(rho, P, slot, n)
    return out


def _angles_for_batch(circuit, node, angles):
    trainable = list(circuit.trainable_nodes)
    if node in trainable:
        return angles[:, trainable.index(node)]
    return np.full(angles.shape[0], circuit[node].angle, dtype=float)


def _initial_batch(circuit, sched, w, inputs, B):
    n_in = len(circuit.input_nodes)
    if inputs is None:
        inputs = np.ones((1, 2**n_in), dtype=complex) / np.sqrt(2**n_in)
    inputs = np.asarray(inputs, dtype=complex).reshape(-1, 2**n_in)
    vec = np.broadcast_to(inputs, (B, 2**n_in)).copy()
    vec = _perm_state_batch(vec, list(circuit.input_nodes), sched[:n_in])
    for _ in range(w - n_in):
        vec = np.einsum("bi,j->bij", vec, _PLUS).reshape(B, -1)
    win = sched[:w]
    g = circuit.graph
    for a, na in enumerate(win):
        for nb in g.neighbors(na):
            if nb in win and na < nb:
                vec = vec * _cz_sign(w, a, win.index(nb))[None]
    return vec


def run_sv_batch(circuit, angles, inputs=None, window_size=1, schedule=None):
    """``run_sv(..., output_form="sv")`` for every row of ``angles`` [B, A]
    with ``inputs`` [B or 1, 2^n_in] (None: |+>).  Returns ``(states [B,
    2^n_out], probs [B, M])``."""
    sched, meas, w = schedule_for(circuit, "sv", window_size, schedule)
    angles = np.atleast_2d(np.asarray(angles, dtype=float))
    B = angles.shape[0]
    if angles.shape[1] != len(circuit.trainable_nodes):
        raise ValueError("Number of angles does not match number of trainable nodes.")
    N = circuit.graph.number_of_nodes()
    psi = _initial_batch(circuit, sched, w, inputs, B)
    probs = np.empty((B, len(meas)))
    g = circuit.graph
    for k, node in enumerate(meas):
        ment = circuit[node]
        n_cur = min(w, N - k)
        p0, _ = _povm_batch(ment.plane, _angles_for_batch(circuit, node, angles))
        proj = _op_on_batch(psi, p0, 0, n_cur)
        probs[:, k] = _re_dot(psi, proj)
        with np.errstate(invalid="ignore", divide="ignore"):
            psi = proj / np.sqrt(_re_dot(proj, proj))[:, None]
            psi = psi.reshape(B, 2, -1).sum(axis=1)
            psi = psi / np.sqrt(_re_dot(psi, psi))[:, None]
        if k + 1 + w <= N:
            win = sched[k + 1 : k + 1 + w]
            sign = np.ones(2**w)
            for nb in g.neighbors(win[-1]):
                if nb in win:
                    sign = sign * _cz_sign(w, win.index(nb), w - 1)
            # psi (x) |+>, then the CZs of the entering qubit
            psi = (psi[:, :, None] * _PLUS[None, None, :]).reshape(B, -1) * sign[None]
    M = len(meas)
    n_cur = min(w, N - M)
    for i in circuit.output_nodes:
        ment = circuit[i]
        if ment is not None and i < n_cur:
            p0, _ = povm(ment.plane, ment.angle)
            psi = _op_on_batch(psi, np.broadcast_to(p0, (B, 2, 2)), i, n_cur)
            psi = psi / np.linalg.norm(psi, axis=1, keepdims=True)
    current = sched[M : M + w]
    if list(circuit.quantum_output_nodes) != current:
        psi = _perm_state_batch(psi, current, list(circuit.output_nodes))
    return psi, probs


def run_dm_batch(circuit, angles, inputs=None, window_size=1, schedule=None, noise_p=0.0):
    """``run_dm`` (mode "sample", no Z-basis steps) for every row of
    ``angles`` [B, A] with pure ``inputs`` [B or 1, 2^n_in].  Returns ``(rho
    [B, d, d], outcomes [B, M] int8, probs [B, M])``; rows whose state turned
    NaN (where the reference raises ValueError) are NaN."""
    sched, meas, w = schedule_for(circuit, "dm", window_size, schedule)
    angles = np.atleast_2d(np.asarray(angles, dtype=float))
    B = angles.shape[0]
    if angles.shape[1] != len(circuit.trainable_nodes):
        raise ValueError("Number of angles does not match number of trainable nodes.")
    if any(circuit[n].plane == "Z" for n in meas):
        raise ValueError("run_dm_batch: Z-basis steps draw outcomes; use run_dm")
    N = circuit.graph.number_of_nodes()
    psi = _initial_batch(circuit, sched, w, inputs, B)
    rho = np.einsum("bi,bj->bij", psi, psi.conj())
    g = circuit.graph
    outcomes = np.zeros((B, len(meas)), dtype=np.int8)
    probs = np.empty((B, len(meas)))
    for k, node in enumerate(meas):
        ment = circuit[node]
        n_cur = min(w, N - k)
        d = 2**n_cur
        rho = _depolarise_slot_batch(rho, 0, n_cur, noise_p)
        p0, p1 = _povm_batch(ment.plane, _angles_for_batch(circuit, node, angles))
        r4 = rho.reshape(B, 2, d // 2, 2, d // 2)
        # Tr(rho (P kron I)) = sum_ab P[b, a] Tr_rest(rho[a, :, b, :])
        blk = np.einsum("bxiyi->bxy", r4)
        prob0 = np.real(np.einsum("bxy,byx->b", blk, p0))
        prob1 = np.real(np.einsum("bxy,byx->b", blk, p1))
        probs[:, k] = prob0
        one = prob0 < 1e-4
        outcomes[:, k] = one
        P = np.where(one[:, None, None], p1, p0)
        pr = np.where(one, prob1, prob0)
        with np.errstate(invalid="ignore", divide="ignore"):
            rho = _sandwich_batch(rho, P, 0, n_cur) / pr[:, None, None]
        t = rho.reshape(B, 2, d // 2, 2, d // 2)
        rho = t[:, 0, :, 0, :] + t[:, 1, :, 1, :]
        if k + 1 + w <= N:
            rho = np.einsum("bij,kl->bikjl", rho, np.full((2, 2), 0.5)).reshape(B, d, d)
            win = sched[k + 1 : k + 1 + w]
            for nb in g.neighbors(win[-1]):
                if nb in win:
                    s = _cz_sign(w, win.index(nb), w - 1)
                    rho = rho * np.outer(s, s)[None]
    M = len(meas)
    n_cur = min(w, N - M)
    for slot in range(n_cur):
        rho = _depolarise_slot_batch(rho, slot, n_cur, noise_p)
    current = [i for i in sched if i not in meas]
    if list(circuit.quantum_output_nodes) != current:
        rho = _perm_rho_batch(rho, current, list(circuit.quantum_output_nodes))
    return rho, outcomes, probs
