"""Shared test helpers: golden fixtures, circuits from specs, and a complex128
interpreter of the window plan (the kernels' in-place conventions on the CPU)."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

from mentpy_gb300.circuit import GraphState, MBQCircuit, Ment
from mentpy_gb300.plan import DEAD

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    spec = json.loads(str(z["spec"]))
    data = {k: z[k] for k in z.files if k != "spec"}
    return spec, data


def circuit_from_spec(spec) -> MBQCircuit:
    g = GraphState()
    g.add_nodes_from(spec["nodes"])
    g.add_edges_from([tuple(e) for e in spec["edges"]])
    meas = {}
    for node, plane, angle in spec["measurements"]:
        meas[node] = None if plane is None else Ment(angle, plane)
    return MBQCircuit(g, spec["input_nodes"], spec["output_nodes"], measurements=meas)


def haar_states(rng, n_qubits, count):
    """Haar-random pure states: normalised complex Gaussian vectors (the
    first column of a Haar unitary has this law), O(2^n) per state."""
    d = 2**n_qubits
    z = rng.standard_normal((count, d)) + 1j * rng.standard_normal((count, d))
    return np.ascontiguousarray(z / np.linalg.norm(z, axis=1, keepdims=True))


def _projector(plane, theta):
    n = {
        0: (np.cos(theta), np.sin(theta), 0.0),
        1: (1.0, 0.0, 0.0),
        2: (0.0, 1.0, 0.0),
        3: (np.cos(theta), 0.0, np.sin(theta)),
        4: (0.0, np.cos(theta), np.sin(theta)),
    }[plane]
    X = np.array([[0, 1], [1, 0]], complex)
    Y = np.array([[0, -1j], [1j, 0]], complex)
    Z = np.array([[1, 0], [0, -1]], complex)
    M = n[0] * X + n[1] * Y + n[2] * Z
    return (np.eye(2) + M) / 2, (np.eye(2) - M) / 2


def _popc(a):
    a = np.asarray(a, dtype=np.int64)
    c = np.zeros_like(a)
    while np.any(a):
        c += a & 1
        a = a >> 1
    return c


def _initial_window(plan, psi_in):
    w, n_in = plan.window, plan.n_in
    idx = np.arange(2**w)
    x = np.zeros_like(idx)
    for i, b in enumerate(plan.in_bits):
        x |= ((idx >> int(b)) & 1) << (n_in - 1 - i)
    psi = np.asarray(psi_in, complex)[x] * 2.0 ** (-(w - n_in) / 2)
    par = np.zeros_like(idx)
    for q in range(w):
        par ^= ((idx >> q) & 1) & (_popc(idx & int(plan.init_cz[q])) & 1)
    return psi * np.where(par, -1.0, 1.0)


def _out_index(plan):
    n = plan.n_out
    y = np.arange(2**n)
    phys = np.zeros_like(y)
    for j, b in enumerate(plan.out_bits):
        phys |= ((y >> (n - 1 - j)) & 1) << int(b)
    return phys


def exec_plan_sv(plan, angles, psi_in, ref_phase=True):
    """Run a statevector plan exactly as the kernels do, in complex128."""
    w = plan.window
    idx = np.arange(2**w)
    psi = _initial_window(plan, psi_in)
    phase = 1.0 + 0j
    for k in range(plan.n_steps):
        p = k % w
        a = int(plan.step_angle[k])
        theta = angles[a] if a >= 0 else plan.step_fixed_angle[k]
        P0, _ = _projector(int(plan.step_plane[k]), theta)
        v = np.array([np.sqrt(P0[0, 0].real), P0[1, 0] / np.sqrt(P0[0, 0].real)])
        c = v.conj()
        lo = idx[((idx >> p) & 1) == 0]
        hi = lo | (1 << p)
        phi = c[0] * psi[lo] + c[1] * psi[hi]
        m = int(plan.step_mask[k])
        psi[lo] = phi
        if m & DEAD:
            psi[hi] = 0
        else:
            psi[hi] = phi * np.where(_popc(hi & m) & 1, -1.0, 1.0)
        s = v[0] + v[1]
        phase *= s / abs(s)
    out = psi[_out_index(plan)]
    out = out / np.linalg.norm(out)
    if ref_phase:
        out = out * phase
    return out


def exec_plan_dm(plan, angles, psi_in, noise_p=0.0):
    """Run a density-matrix plan as the kernels do; returns (rho, outcomes, probs)."""
    w = plan.window
    d = 2**w
    psi = _initial_window(plan, psi_in)
    rho = np.outer(psi, psi.conj())
    # the initial window carries the padding |+> amplitudes; the reference
    # trace is |psi_in|^2
    idx = np.arange(d)
    outcomes, probs = [], []
    a_, b_ = 1 - 4 * noise_p / 3, 2 * noise_p / 3
    for k in range(plan.n_steps):
        p = k % w
        a = int(plan.step_angle[k])
        theta = angles[a] if a >= 0 else plan.step_fixed_angle[k]
        P0, P1 = _projector(int(plan.step_plane[k]), theta)
        lo = idx[((idx >> p) & 1) == 0]
        hi = lo | (1 << p)
        blk = {(x, y): rho[np.ix_(lo if x == 0 else hi, lo if y == 0 else hi)] for x in (0, 1) for y in (0, 1)}

        def contract(P):
            s = sum(P[y, x] * blk[(x, y)] for x in (0, 1) for y in (0, 1))
            return a_ * s + b_ * (blk[(0, 0)] + blk[(1, 1)])

        sig0 = contract(P0)
        prob0 = float(np.real(np.trace(sig0)))
        probs.append(prob0)
        if prob0 < 1e-4:
            sig = contract(P1)
            prob = float(np.real(np.trace(sig)))
            outcomes.append(1)
        else:
            sig, prob = sig0, prob0
            outcomes.append(0)
        sig = sig / prob
        m = int(plan.step_mask[k])
        new = np.zeros_like(rho)
        if m & DEAD:
            new[np.ix_(lo, lo)] = sig
        else:
            s = np.where(_popc(hi & m) & 1, -1.0, 1.0)
            new[np.ix_(lo, lo)] = sig / 2
            new[np.ix_(lo, hi)] = sig * s[None, :] / 2
            new[np.ix_(hi, lo)] = sig * s[:, None] / 2
            new[np.ix_(hi, hi)] = sig * np.outer(s, s) / 2
        rho = new
    oi = _out_index(plan)
    out = rho[np.ix_(oi, oi)]
    if noise_p:
        n = plan.n_out
        for j in range(n):
            t = out.reshape(2**j, 2, 2 ** (n - j - 1), 2**j, 2, 2 ** (n - j - 1))
            diag = t[:, 0, :, :, 0, :] + t[:, 1, :, :, 1, :]
            t = a_ * t
            t[:, 0, :, :, 0, :] += b_ * diag
            t[:, 1, :, :, 1, :] += b_ * diag
            out = t.reshape(2**n, 2**n)
    return out, outcomes, probs


def exec_plan_sv_adjoint(plan, angles, psi_in, grad_out):
    """The adjoint kernel's math in complex128: dL/dangles for
    dL = Re <grad_out|dz>, z the canonical (phase-free) normalised output."""
    w = plan.window
    idx = np.arange(2**w)
    psi = _initial_window(plan, psi_in).astype(complex)
    hist, coefs = [], []
    for k in range(plan.n_steps):
        p = k % w
        a = int(plan.step_angle[k])
        theta = angles[a] if a >= 0 else plan.step_fixed_angle[k]
        plane = int(plan.step_plane[k])
        theta_eff = {0: theta, 1: 0.0, 2: np.pi / 2}[plane]
        c = np.exp(-1j * theta_eff)
        lo = idx[((idx >> p) & 1) == 0]
        hi = lo | (1 << p)
        hist.append(psi[hi].copy())
        coefs.append(c)
        phi = psi[lo] + c * psi[hi]
        m = int(plan.step_mask[k])
        psi = psi.copy()
        psi[lo] = phi
        psi[hi] = 0 if (m & DEAD) else phi * np.where(_popc(hi & m) & 1, -1.0, 1.0)
    oi = _out_index(plan)
    n = np.linalg.norm(psi)
    z = psi[oi] / n
    g = np.asarray(grad_out, complex)
    lam = np.zeros_like(psi)
    lam[oi] = (g - np.real(np.vdot(z, g)) * z) / n
    grad = np.zeros(plan.n_angles)
    for k in range(plan.n_steps - 1, -1, -1):
        p = k % w
        lo = idx[((idx >> p) & 1) == 0]
        hi = lo | (1 << p)
        m = int(plan.step_mask[k])
        mu = lam[lo] if (m & DEAD) else lam[lo] + np.where(_popc(hi & m) & 1, -1.0, 1.0) * lam[hi]
        c = coefs[k]
        t = np.sum(np.conj(mu) * hist[k])
        a = int(plan.step_angle[k])
        if a >= 0:
            grad[a] += np.imag(c * t)
        lam = lam.copy()
        lam[lo] = mu
        lam[hi] = np.conj(c) * mu
    return grad


def exec_plan_dm_factored(plan, angles, psi_in, noise_p=0.0):
    """The factored density-matrix recurrence of csrc/dm_fact.cuh in
    complex128: only R, the matrix over the window bits other than the slot
    of the last entering qubit, is kept; that slot's |+> (or |0>) and CZ
    signs are applied implicitly.  Returns (rho, outcomes, probs) like
    ``exec_plan_dm``."""
    w = plan.window
    M = plan.n_steps
    assert w >= 2 and M >= 1 and (int(plan.step_mask[M - 1]) & DEAD)
    D = 2 ** (w - 1)
    psi = _initial_window(plan, psi_in)
    a_n, b_n = 1 - 4 * noise_p / 3, 2 * noise_p / 3
    tr_noise = a_n + 2 * b_n

    def functional(k):
        a = int(plan.step_angle[k])
        theta = angles[a] if a >= 0 else plan.step_fixed_angle[k]
        P0, _ = _projector(int(plan.step_plane[k]), theta)
        # G[a, b]: coefficient of rho[(a, r), (b, r')] in the contraction
        return a_n * P0.T + b_n * np.eye(2)

    def ins(r, pos, b):
        return ((r >> pos) << (pos + 1)) | (b << pos) | (r & ((1 << pos) - 1))

    pos_of = {0: None}
    pos_of.update({b: b - 1 for b in range(1, w)})
    p, pmask = 0, int(plan.step_mask[0])
    outcomes, probs = [], []
    R = None
    for k in range(M):
        G = functional(k)
        if k == 0:
            x0, x1 = psi[0::2], psi[1::2]
            blocks = {(0, 0): np.outer(x0, x0.conj()), (0, 1): np.outer(x0, x1.conj()),
                      (1, 0): np.outer(x1, x0.conj()), (1, 1): np.outer(x1, x1.conj())}
            drop_coh, dead, mq, pos, sgn = False, False, False, None, 0
        else:
            q = k % w
            pos = pos_of[q]
            dead = bool(pmask & DEAD)
            mq = (not dead) and bool((pmask >> q) & 1)
            sgn = 0
            if not dead:
                for b in range(w):
                    if b not in (p, q) and (pmask >> b) & 1:
                        sgn |= 1 << pos_of[b]
            H = D // 2
            rr = np.arange(H)
            i0, i1 = ins(rr, pos, 0), ins(rr, pos, 1)
            blocks = {(a, b): R[np.ix_(i0 if a == 0 else i1, i0 if b == 0 else i1)] for a in (0, 1) for b in (0, 1)}
            drop_coh = (not dead) and mq

        def trace_of(Gm):
            d = sum(Gm[a, b] * np.trace(blocks[(a, b)]) for a in (0, 1) for b in (0, 1) if a == b or not drop_coh)
            return float(np.real(d))

        prob0 = trace_of(G)
        probs.append(prob0)
        if prob0 < 1e-4:
            G = tr_noise * np.eye(2) - G
            prob, outc = trace_of(G), 1
        else:
            prob, outc = prob0, 0
        outcomes.append(outc)
        P = {(a, b): G[a, b] * blocks[(a, b)] for a in (0, 1) for b in (0, 1)}
        if k == 0:
            R = sum(P.values()) / prob
        else:
            T = {}
            for ap in (0, 1):
                for bp in (0, 1):
                    T[(ap, bp)] = sum(P[(a, b)] * (-1.0) ** ((ap * a + bp * b) * int(mq)) for a in (0, 1) for b in (0, 1))
            pi = np.array([bin(int(x) & sgn).count("1") & 1 for x in i0])
            new = np.zeros_like(R)
            for ap in (0, 1):
                for bp in (0, 1):
                    if dead and (ap or bp):
                        continue
                    f = 1.0 if dead else 0.5
                    s = (-1.0) ** (ap * pi)[:, None] * (-1.0) ** (bp * pi)[None, :]
                    new[np.ix_(i0 if ap == 0 else i1, i0 if bp == 0 else i1)] = f * s * T[(ap, bp)] / prob
            R = new
            pos_of[p] = pos
            pos_of[q] = None
            p = q
        pmask = int(plan.step_mask[k])
    # output noise on the output positions, then the gather in the reference order
    n = plan.n_out
    for j in range(n):
        pos = pos_of[int(plan.out_bits[j])]
        H = D // 2
        rr = np.arange(H)
        i0, i1 = ins(rr, pos, 0), ins(rr, pos, 1)
        x00, x11 = R[np.ix_(i0, i0)].copy(), R[np.ix_(i1, i1)].copy()
        tr = x00 + x11
        R[np.ix_(i0, i0)] = a_n * x00 + b_n * tr
        R[np.ix_(i1, i1)] = a_n * x11 + b_n * tr
        R[np.ix_(i0, i1)] *= a_n
        R[np.ix_(i1, i0)] *= a_n
    y = np.arange(2**n)
    ridx = np.zeros_like(y)
    for j in range(n):
        ridx |= ((y >> (n - 1 - j)) & 1) << pos_of[int(plan.out_bits[j])]
    return R[np.ix_(ridx, ridx)], outcomes, probs
