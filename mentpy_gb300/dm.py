"""Density-matrix sweeps on the GPU: the ``cuda-dm`` backend and uneven batches.

``DensityMatrixSweep`` runs batches of mentpy's density-matrix sweep
(np_simulator_dm.py:218-346) in one launch; ``UnevenDensityMatrixBatch`` runs
many different circuits (different widths and depths) together: the circuits
share one device plan table, runs are grouped by window size into one kernel
launch per size, and the launches go to separate streams (or one CUDA graph)
so that small and large windows occupy the GPU at the same time.
``CudaSimulatorDM`` is the drop-in for ``NumpySimulatorDM``.
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _native
from .plan import DEAD, PLANE_CODES, WindowPlan, compile_plan
from .simulators import BaseSimulator, _pop_kwargs
from .sweep import _ptr, _stream_ptr, as_device

DM_MAX_WINDOW = 11     # forward (factored kernels; windows 9..11 through a workspace)
DM_BATCH_MAX_WINDOW = 8  # uneven batches (shared-memory kernels)
DM_ADJ_MAX_WINDOW = 10  # adjoint through the channel (windows 8..10 through a workspace)
NAN_MESSAGE = "qstate has nan, you might want to increase the window size"


class DensityMatrixSweep:
    """Batched density-matrix sweep of one circuit (complex64, FP64 outcome
    probabilities)."""

    def __init__(self, circuit=None, window_size: int = 1, schedule=None, *, plan: Optional[WindowPlan] = None,
                 device=None):
        if plan is None:
            plan = compile_plan(circuit, "dm", window_size=window_size, schedule=schedule)
        if plan.kind != "dm":
            raise ValueError("DensityMatrixSweep needs a density-matrix plan")
        if plan.window > DM_MAX_WINDOW:
            raise NotImplementedError(f"density-matrix window {plan.window} > {DM_MAX_WINDOW}")
        self.plan = plan
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dplan = _native.DevicePlan(plan)
        self.n_in, self.n_out, self.n_angles = plan.n_in, plan.n_out, plan.n_angles
        self.has_z = bool((np.asarray(plan.step_plane) == PLANE_CODES["Z"]).any())

    def forward(self, angles, inputs=None, *, noise: float = 0.0, want_probs: bool = False, stream=None,
                mode: str = "sample", seed: Optional[int] = None, full_matrix: bool = False):
        """Returns ``(rho [B, d, d], outcomes [B, M] int8, status [B], probs)``.

        ``mode`` as ``NumpySimulatorDM.run``: Z-basis steps draw their outcome
        ("sample", from ``seed``; default: a draw from numpy's global
        generator, as the reference draws from it) or, with "expectation" /
        "exp", trace the qubit out unprojected and record prob1 / (prob0 +
        prob1) (``outcomes`` 2 and the value in ``probs``).  Other steps keep
        the reference's rule (outcome 1 iff prob0 < 1e-4).  ``full_matrix``
        keeps the whole 2^w x 2^w matrix (windows <= 7) instead of the
        factored form (same results to float rounding)."""
        if mode not in ("sample", "expectation", "exp"):
            raise ValueError(f"unknown mode {mode!r}")
        flags = _native.MBQC_F_DM_EXPECTATION if mode in ("expectation", "exp") else 0
        if full_matrix:
            flags |= _native.MBQC_F_DM_FULL_MATRIX
        if seed is None:
            seed = int(np.random.randint(0, 2**63 - 1, dtype=np.int64)) if self.has_z else 0
        ang = as_device(angles, torch.float64, self.device)
        if ang.dim() == 1:
            ang = ang.unsqueeze(0)
        B = ang.shape[0]
        if ang.shape[1] != self.n_angles:
            raise ValueError(
                f"Number of angles ({ang.shape[1]}) does not match number of trainable nodes ({self.n_angles})."
            )
        if inputs is None:
            d = 2 ** self.n_in
            inp = torch.full((1, d), 1.0 / np.sqrt(d), dtype=torch.complex64, device=self.device)
        else:
            inp = as_device(inputs, torch.complex64, self.device)
            if inp.dim() == 1:
                inp = inp.unsqueeze(0)
        istride = 0 if inp.shape[0] == 1 else inp.shape[1]
        d_out = 2 ** self.n_out
        M = self.plan.n_steps
        rho = torch.empty((B, d_out, d_out), dtype=torch.complex64, device=self.device)
        outc = torch.empty((B, max(M, 1)), dtype=torch.int8, device=self.device)
        status = torch.empty((B,), dtype=torch.int32, device=self.device)
        probs = torch.empty((B, max(M, 1)), dtype=torch.float64, device=self.device) if want_probs else None
        L = _native.lib()
        n = ctypes.c_size_t()
        _native.check(L.mbqc_dm_forward_workspace(self.dplan.handle, B, self.plan.window, ctypes.byref(n)))
        ws = None
        if n.value:
            ws = getattr(self, "_fws", None)
            if ws is None or ws.numel() < n.value:
                ws = torch.empty(n.value, dtype=torch.uint8, device=self.device)
                self._fws = ws
        _native.check(L.mbqc_dm_forward_ws(
            self.dplan.handle, B, self.plan.window, None, _ptr(ang), max(ang.shape[1], 1), _ptr(inp), istride,
            _ptr(rho), d_out * d_out, float(noise), _ptr(outc), _ptr(probs), max(M, 1), _ptr(status), flags,
            int(seed) & (2**64 - 1), _ptr(ws), 0 if ws is None else ws.numel(), _stream_ptr(stream)))
        return rho, outc[:, :M], status, (probs[:, :M] if probs is not None else None)

    def adjoint(self, angles, inputs, grad_out, *, noise: float = 0.0, stream=None):
        """dL/dangles [B, A] (float64) for dL = Re sum conj(grad_out) d rho_out,
        through the noisy channel with the outcomes of this forward pass held
        fixed.  Returns ``(grad, rho, status)``."""
        ang = as_device(angles, torch.float64, self.device)
        if ang.dim() == 1:
            ang = ang.unsqueeze(0)
        B = ang.shape[0]
        if inputs is None:
            d = 2 ** self.n_in
            inp = torch.full((1, d), 1.0 / np.sqrt(d), dtype=torch.complex64, device=self.device)
        else:
            inp = as_device(inputs, torch.complex64, self.device)
            if inp.dim() == 1:
                inp = inp.unsqueeze(0)
        istride = 0 if inp.shape[0] == 1 else inp.shape[1]
        d_out = 2 ** self.n_out
        g = as_device(grad_out, torch.complex64, self.device).reshape(B, d_out * d_out)
        rho = torch.empty((B, d_out, d_out), dtype=torch.complex64, device=self.device)
        grad = torch.empty((B, max(self.n_angles, 1)), dtype=torch.float64, device=self.device)
        status = torch.empty((B,), dtype=torch.int32, device=self.device)
        L = _native.lib()
        n = ctypes.c_size_t()
        _native.check(L.mbqc_dm_adjoint_workspace(self.dplan.handle, B, self.plan.window, None, ctypes.byref(n)))
        ws = getattr(self, "_ws", None)
        if ws is None or ws.numel() < n.value:
            ws = torch.empty(max(n.value, 16), dtype=torch.uint8, device=self.device)
            self._ws = ws
        _native.check(L.mbqc_dm_adjoint(
            self.dplan.handle, B, self.plan.window, None, _ptr(ang), max(ang.shape[1], 1), _ptr(inp), istride,
            float(noise), _ptr(g), d_out * d_out, _ptr(rho), d_out * d_out, _ptr(grad), max(self.n_angles, 1),
            None, 1, _ptr(status), _ptr(ws), ws.numel(), _stream_ptr(stream)))
        return grad[:, : self.n_angles], rho, status


class _DmFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, angles, inputs, sweep, noise):
        rho, _, _, _ = sweep.forward(angles.detach(), inputs, noise=noise)
        ctx.sweep, ctx.inputs, ctx.noise = sweep, inputs, noise
        ctx.save_for_backward(angles)
        return rho

    @staticmethod
    def backward(ctx, grad_rho):
        (angles,) = ctx.saved_tensors
        g, _, _ = ctx.sweep.adjoint(angles.detach(), ctx.inputs, grad_rho.contiguous(), noise=ctx.noise)
        return g.to(angles.dtype), None, None, None


def dm_states(sweep: "DensityMatrixSweep", angles: torch.Tensor, inputs=None, noise: float = 0.0) -> torch.Tensor:
    """Output density matrices [B, d, d] of the (noisy) density-matrix sweep,
    differentiable with respect to ``angles`` through the channel (outcomes
    held fixed, as the reference's bookkeeping fixes them)."""
    if angles.dim() == 1:
        angles = angles.unsqueeze(0)
    return _DmFunction.apply(angles, inputs, sweep, noise)


_DM_TILE_SHAPES = {2: (32,), 3: (32,), 4: (32,), 5: (32, 64), 6: (32, 64, 128), 7: (64, 128, 256), 8: (256,)}
_DM_TUNED = {}  # batch signature -> (tile threads per window, blocks per SM, long-circuit tile threads)
_DM_LONG_QUANTILE = 0.8  # circuits at or above this quantile of their window's step counts are "long"


def _factorable(p) -> bool:
    """The factored kernel takes windows 2..8 whose last step shrinks the
    window; the shrinking steps are the last w - n_out, so that is w > n_out
    (also for the shape-only plans of the native batch compiler)."""
    if not (2 <= p.window <= 8 and p.n_steps >= 1 and p.window > p.n_out):
        return False
    mask = getattr(p, "step_mask", None)
    return mask is None or bool(int(mask[-1]) & DEAD)


class _NativeDmBatch:
    """Owner of one mbqc_dm_batch (tile schedule on the device)."""

    def __init__(self, dplan, n, tpr, blocks_per_sm, long_tpr=None, long_steps=None):
        arr = (ctypes.c_int32 * 9)(*[int(tpr.get(w, 0)) for w in range(9)])
        ltpr = (ctypes.c_int32 * 9)(*[int((long_tpr or {}).get(w, 0)) for w in range(9)])
        lsteps = (ctypes.c_int32 * 9)(*[int((long_steps or {}).get(w, 0)) for w in range(9)])
        h = ctypes.c_void_p()
        _native.check(_native.lib().mbqc_dm_batch_create_ex(dplan.handle, n, arr, ltpr, lsteps, int(blocks_per_sm),
                                                             ctypes.byref(h)))
        self.handle = h
        self._dplan = dplan  # the schedule refers to the plan table
        info = (ctypes.c_int32 * 10)()
        _native.check(_native.lib().mbqc_dm_batch_info(h, info))
        self.n_tiles, self.blocks, self.smem = int(info[0]), int(info[1]), int(info[2])
        self.tpr = {w: int(info[1 + w]) for w in range(2, 9)}

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _native is not None:
            try:
                _native.lib().mbqc_dm_batch_destroy(h)
            except Exception:
                pass


class UnevenDensityMatrixBatch:
    """Many circuits of different widths and depths, one run each per call.

    All plans live in one device plan table.  By default the whole batch is
    ONE persistent kernel launch (``mbqc_dm_batch_forward``): runs are cut
    into tiles of one window (the tile shape -- threads per run -- per
    window from ``tune()``), ordered longest first, and the resident blocks
    claim tiles until none is left.  ``persistent=False`` (or circuits the
    factored kernel does not take) groups the runs by window size instead,
    one launch per size on its own stream.  ``capture()`` records a call into
    a CUDA graph.
    """

    def __init__(self, plans: Sequence[WindowPlan], device=None, *, _dplan=None, persistent: bool = True):
        self.plans = list(plans)
        for p in self.plans:
            if p.kind != "dm" or p.window > DM_BATCH_MAX_WINDOW:
                raise ValueError(f"density-matrix plans with window <= {DM_BATCH_MAX_WINDOW} expected")
        self.persistent = bool(persistent) and all(_factorable(p) for p in self.plans)
        self._nbatch = None
        sig = tuple(sorted((p.window, p.n_steps) for p in self.plans))
        self._sig = (len(self.plans), hash(sig))
        self.tile_tpr, self.blocks_per_sm, self.long_tpr = _DM_TUNED.get(self._sig, ({}, 0, {}))
        # per window: the step count from which a circuit is "long" (it may take
        # its own tile shape, set by tune())
        steps_by_w: Dict[int, List[int]] = {}
        for p in self.plans:
            steps_by_w.setdefault(p.window, []).append(p.n_steps)
        self.long_steps = {w: int(np.quantile(v, _DM_LONG_QUANTILE, method="higher"))
                           for w, v in steps_by_w.items() if len(v) >= 8}
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dplan = _dplan if _dplan is not None else _native.DevicePlan(self.plans)
        self.max_a = max(max(p.n_angles for p in self.plans), 1)
        self.max_in = max(p.n_in for p in self.plans)
        self.max_out = max(p.n_out for p in self.plans)
        self.max_m = max(max(p.n_steps for p in self.plans), 1)
        # groups by window, largest work first
        groups: Dict[int, List[int]] = {}
        for i, p in enumerate(self.plans):
            groups.setdefault(p.window, []).append(i)
        self.groups = []
        for w in sorted(groups, reverse=True):
            idx = sorted(groups[w], key=lambda i: -self.plans[i].n_steps)
            self.groups.append((w, torch.tensor(idx, dtype=torch.int32, device=self.device)))
        self.streams = [torch.cuda.Stream(device=self.device) for _ in self.groups]
        self._graph = None

    @classmethod
    def from_graph_batch(cls, batch, device=None) -> "UnevenDensityMatrixBatch":
        """Compile a ``native_plan.GraphBatch`` (thousands of open graphs in
        flat arrays) natively and upload it as one plan table -- no
        ``MBQCircuit`` objects, milliseconds for thousands of circuits."""
        from .native_plan import compile_graph_batch

        dplan, infos = compile_graph_batch(batch, "dm")
        return cls(infos, device=device, _dplan=dplan)

    def allocate(self):
        """Device buffers for one call: angles [C, max_a] (float64), inputs
        [C, 2^max_in], rho [C, 4^max_out], outcomes/probs [C, max_m], status [C]."""
        C = len(self.plans)
        dev = self.device
        return dict(
            angles=torch.zeros((C, self.max_a), dtype=torch.float64, device=dev),
            inputs=torch.zeros((C, 2 ** self.max_in), dtype=torch.complex64, device=dev),
            rho=torch.zeros((C, 4 ** self.max_out), dtype=torch.complex64, device=dev),
            outcomes=torch.zeros((C, self.max_m), dtype=torch.int8, device=dev),
            probs=torch.zeros((C, self.max_m), dtype=torch.float64, device=dev),
            status=torch.zeros((C,), dtype=torch.int32, device=dev),
        )

    def native_batch(self) -> "_NativeDmBatch":
        """The device tile schedule for the current tile shapes."""
        if self._nbatch is None:
            self._nbatch = _NativeDmBatch(self.dplan, len(self.plans), self.tile_tpr, self.blocks_per_sm,
                                          self.long_tpr, self.long_steps)
        return self._nbatch

    def _launch_all(self, buf, noise):
        if self.persistent:
            nb = self.native_batch()
            _native.check(_native.lib().mbqc_dm_batch_forward(
                nb.handle, _ptr(buf["angles"]), self.max_a, _ptr(buf["inputs"]), 2 ** self.max_in,
                _ptr(buf["rho"]), 4 ** self.max_out, float(noise), _ptr(buf["outcomes"]), _ptr(buf["probs"]),
                self.max_m, _ptr(buf["status"]), 0, 0, _stream_ptr(None)))
            return
        main = torch.cuda.current_stream(self.device)
        L = _native.lib()
        for (w, idx), s in zip(self.groups, self.streams):
            s.wait_stream(main)
            _native.check(L.mbqc_dm_forward(
                self.dplan.handle, idx.numel(), w, _ptr(idx), _ptr(buf["angles"]), self.max_a, _ptr(buf["inputs"]),
                2 ** self.max_in, _ptr(buf["rho"]), 4 ** self.max_out, float(noise), _ptr(buf["outcomes"]),
                _ptr(buf["probs"]), self.max_m, _ptr(buf["status"]), _stream_ptr(s)))
        for s in self.streams:
            main.wait_stream(s)

    def run(self, buf, noise: float = 0.0):
        """One call over all circuits: reads buf['angles'], buf['inputs'] (row
        c = circuit c), writes buf['rho'], buf['outcomes'], buf['probs'],
        buf['status'].  Replays the captured graph when it matches."""
        if self._graph is not None and self._graph_buf is buf and self._graph_noise == noise:
            self._graph.replay()
        else:
            self._launch_all(buf, noise)
        return buf

    def tune(self, buf, noise: float = 0.0, reps: int = 5) -> dict:
        """Autotune the persistent launch on this batch: for every window
        present, the tile shape (threads per run, hence runs per block) by
        coordinate descent from the defaults, then the shape of the window's
        longest circuits (the top fifth by steps, which end the batch), then
        the resident blocks per SM; each candidate is timed (CUDA events,
        ``reps`` launches after a warm-up).  The choice is cached per batch
        composition and used by later batches of the same circuits.  Returns
        the choice and the timings."""
        if not self.persistent:
            return {}
        windows = sorted({p.window for p in self.plans})
        long_tpr = {}

        def timed(tpr, bps, ltpr=None):
            self.tile_tpr, self.blocks_per_sm, self._nbatch = dict(tpr), bps, None
            self.long_tpr = dict(long_tpr if ltpr is None else ltpr)
            self._graph = None
            for _ in range(2):
                self._launch_all(buf, noise)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            from .sweep import gpu_hold

            gpu_hold(500.0)
            e0.record()
            for _ in range(reps):
                self._launch_all(buf, noise)
            e1.record()
            torch.cuda.synchronize(self.device)
            return e0.elapsed_time(e1) / reps

        best_tpr, best_bps = dict(self.tile_tpr), 0
        best = timed(best_tpr, best_bps)
        log = [(dict(best_tpr), best_bps, best)]
        for w in windows:
            for t in _DM_TILE_SHAPES[w]:
                if best_tpr.get(w, 0) == t:
                    continue
                cand = dict(best_tpr)
                cand[w] = t
                ms = timed(cand, best_bps)
                log.append((dict(cand), best_bps, ms))
                if ms < best:
                    best, best_tpr = ms, cand
        for w in windows:
            if w not in self.long_steps:
                continue
            base = self.native_batch().tpr[w] if best_tpr.get(w, 0) == 0 else best_tpr[w]
            for t in _DM_TILE_SHAPES[w]:
                if t <= base:
                    continue
                cand = dict(long_tpr)
                cand[w] = t
                ms = timed(best_tpr, best_bps, cand)
                log.append((dict(best_tpr), best_bps, ms))
                if ms < best:
                    best, long_tpr = ms, cand
        occ = self.native_batch().blocks // max(1, _native.sm_count())
        for bps in range(1, max(occ, 1)):
            ms = timed(best_tpr, bps)
            log.append((dict(best_tpr), bps, ms))
            if ms < best:
                best, best_bps = ms, bps
        self.tile_tpr, self.blocks_per_sm, self.long_tpr, self._nbatch = best_tpr, best_bps, long_tpr, None
        self._graph = None
        _DM_TUNED[self._sig] = (best_tpr, best_bps, long_tpr)
        return {"tile_threads": {w: self.native_batch().tpr[w] for w in windows}, "blocks_per_sm": best_bps,
                "long_circuit_tile_threads": dict(long_tpr), "long_steps": dict(self.long_steps), "ms": best,
                "candidates": len(log)}

    def capture(self, buf, noise: float = 0.0):
        """Record the per-window launches into one CUDA graph."""
        self._launch_all(buf, noise)  # warm-up outside capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._launch_all(buf, noise)
        self._graph, self._graph_buf, self._graph_noise = g, buf, noise
        return g

    def adjoint(self, buf, noise: float = 0.0):
        """Gradients through the channel for every circuit: reads buf['angles'],
        buf['inputs'] and buf['grad_out'] ([C, 4^max_out], dL/drho_out), writes
        buf['grad'] ([C, max_a]) and the forward outputs, one launch per window
        size on its own stream."""
        dev = self.device
        C = len(self.plans)
        if "grad" not in buf:
            buf["grad"] = torch.zeros((C, self.max_a), dtype=torch.float64, device=dev)
        if "grad_out" not in buf:
            raise KeyError("buf['grad_out'] ([C, 4^max_out] complex64) is required")
        L = _native.lib()
        if not hasattr(self, "_adj_ws"):
            self._adj_ws = {}
            for w, idx in self.groups:
                n = ctypes.c_size_t()
                _native.check(L.mbqc_dm_adjoint_workspace(self.dplan.handle, idx.numel(), w, _ptr(idx),
                                                          ctypes.byref(n)))
                self._adj_ws[w] = torch.empty(max(n.value, 16), dtype=torch.uint8, device=dev)
        main = torch.cuda.current_stream(dev)
        for (w, idx), s in zip(self.groups, self.streams):
            s.wait_stream(main)
            ws = self._adj_ws[w]
            _native.check(L.mbqc_dm_adjoint(
                self.dplan.handle, idx.numel(), w, _ptr(idx), _ptr(buf["angles"]), self.max_a, _ptr(buf["inputs"]),
                2 ** self.max_in, float(noise), _ptr(buf["grad_out"]), 4 ** self.max_out, _ptr(buf["rho"]),
                4 ** self.max_out, _ptr(buf["grad"]), self.max_a, _ptr(buf["outcomes"]), self.max_m,
                _ptr(buf["status"]), _ptr(ws), ws.numel(), _stream_ptr(s)))
        for s in self.streams:
            main.wait_stream(s)
        return buf

    def rho(self, buf, c: int) -> torch.Tensor:
        """Output density matrix of circuit ``c``."""
        d = 2 ** self.plans[c].n_out
        return buf["rho"][c, : d * d].reshape(d, d)


class CudaSimulatorDM(BaseSimulator):
    """GPU density-matrix simulator, drop-in for ``NumpySimulatorDM``
    (np_simulator_dm.py:29-380): ``run(angles, mode="sample", input_state=None)``
    returns rho over the quantum outputs; ``outcomes`` follows the reference's
    rule (1 iff prob0 < 1e-4); a NaN state raises ``ValueError`` like the
    reference.  Extra keyword ``noise``: depolarising strength (default 0)."""

    def __init__(self, mbqcircuit, input_state: np.ndarray = None, **kwargs) -> None:
        super().__init__(mbqcircuit, input_state)
        self.noise = float(kwargs.pop("noise", 0.0))
        o = _pop_kwargs(kwargs)
        self.force0 = o["force0"]
        self.plan = compile_plan(mbqcircuit, "dm", window_size=o["window_size"], schedule=o["schedule"],
                                 force0=o["force0"], dev_mode=o["dev_mode"])
        self.window_size = self.plan.window
        self.schedule = self.plan.schedule
        self.schedule_measure = self.plan.schedule_measure
        self._sweep = DensityMatrixSweep(plan=self.plan, device=o["device"])
        self.current_measurement = 0
        self._qstate = None

    @property
    def qstate(self):
        return self._qstate

    def reset(self, input_state: np.ndarray = None):
        self.current_measurement = 0
        if input_state is not None:
            self.input_state = input_state
        self.outcomes = {}

    def measure(self, angle: float, mode="sample"):
        raise NotImplementedError(
            "the GPU backend executes whole sweeps; call run(angles) instead of measure()"
        )

    def run_batch(self, angles, input_states=None, *, mode: str = "sample", seed: Optional[int] = None,
                  stream=None):
        """B independent runs in one launch: ``angles`` [B, A] (or [A]),
        ``input_states`` [B or 1, 2^n_in], [2^n_in] or None (this
        simulator's input state).  No counterpart in the reference, whose
        ``run`` takes one angle vector (np_simulator_dm.py:218-283); each row
        gives what ``reset(input_state=row)`` + ``run(row angles, mode)``
        gives, and the simulator's own state is left untouched.  Returns a
        ``BatchResult`` (rho [B, d, d], outcomes [B, M] int8 in schedule
        order: 0/1, or 2 for an expectation-mode Z step whose value is in
        ``logprob``'s place, the probs [B, M] array of prob0 per step).  A
        NaN state is reported as ``status`` RUN_NAN for that row (the
        reference raises ValueError on its single run).  numpy inputs give
        numpy results, torch tensors give device tensors."""
        from .simulators import BatchResult

        as_np = not isinstance(angles, torch.Tensor)
        ang = np.asarray(angles, dtype=np.float64) if as_np else angles
        if len(ang.shape) == 1:
            ang = ang.reshape(1, -1)
        if ang.shape[1] != len(self.mbqcircuit.trainable_nodes):
            raise ValueError(
                f"Number of angles ({ang.shape[1]}) does not match number of trainable nodes "
                f"({len(self.mbqcircuit.trainable_nodes)})."
            )
        inp = self.input_state if input_states is None else input_states
        if inp is not None and not isinstance(inp, torch.Tensor):
            inp = np.asarray(inp).reshape(-1, 2 ** self._sweep.n_in)
        rho, outc, status, probs = self._sweep.forward(ang, inp, noise=self.noise, mode=mode, seed=seed,
                                                       want_probs=True, stream=stream)
        if as_np:
            return BatchResult(rho.cpu().numpy().astype(np.complex128), outc.cpu().numpy(), status.cpu().numpy(),
                               probs.cpu().numpy())
        return BatchResult(rho, outc, status, probs)

    def run(self, angles, mode="sample", input_state=None):
        if input_state is not None:
            self.reset(input_state=input_state)
        if len(angles) != len(self.mbqcircuit.trainable_nodes):
            raise ValueError(
                f"Number of angles ({len(angles)}) does not match number of trainable nodes "
                f"({len(self.mbqcircuit.trainable_nodes)})."
            )
        if self.current_measurement >= len(self.schedule_measure):
            raise ValueError("No more measurements to be done.")
        inp = None if self.input_state is None else np.asarray(self.input_state).reshape(1, -1)
        rho, outc, status, probs = self._sweep.forward(np.asarray(angles, dtype=np.float64).reshape(1, -1), inp,
                                                       noise=self.noise, mode=mode, want_probs=True)
        self.current_measurement = len(self.schedule_measure)
        outc = outc[0].cpu().numpy()
        pr = probs[0].cpu().numpy()
        # expectation-mode Z steps record prob1 / (prob0 + prob1) as a float
        # (np_simulator_dm.py:327-331); every other outcome is 0 or 1
        self.outcomes = {node: (float(p) if o == 2 else int(o))
                         for node, o, p in zip(self.schedule_measure, outc, pr)}
        if int(status[0].item()) != _native.RUN_OK:
            raise ValueError(NAN_MESSAGE)
        r = rho[0].cpu().numpy().astype(np.complex128)
        self._qstate = r
        return r
