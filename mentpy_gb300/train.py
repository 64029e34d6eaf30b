"""Whole training runs on the device: fused fidelity adjoint + Adam.

``FidelityTrainer`` trains V angle vectors at once against one data set of J
(input, target) pairs with mentpy's loss 1 - mean_j |<t_j|z_j>|^2
(docs/tutorials/intro-to-mbqml.rst) and mentpy's Adam
(optimizers/adam.py:54-66).  One iteration is one fused adjoint launch over
the V x J runs (``StatevectorSweep.fidelity_grad``) and one Adam step
(``mbqc_adam_step``); the iteration is recorded once into a CUDA graph and
replayed, so a training run makes no host round trip until it ends.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import torch

from . import _native
from .sweep import StatevectorSweep, _ptr, _stream_ptr, as_device

__all__ = ["FidelityTrainer"]


class FidelityTrainer:
    """Train ``angles0`` [V, A] (one row per independent run) on the device.

    ``step_size``, ``b1``, ``b2``, ``eps`` as ``mentpy.optimizers.AdamOptimizer``.
    ``losses`` [n, V] holds the loss at the angles each iteration started
    from (the gradient's point), ``angles`` the current parameters.
    """

    def __init__(self, sweep: StatevectorSweep, inputs, targets, angles0, *, step_size: float = 0.1,
                 b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        dev = sweep.device
        self.sweep = sweep
        self.inputs = as_device(inputs, torch.complex64, dev)
        self.targets = as_device(targets, torch.complex64, dev)
        x = as_device(angles0, torch.float64, dev)
        self.angles = (x.unsqueeze(0) if x.dim() == 1 else x).clone()
        V, A = self.angles.shape
        if A != sweep.n_angles:
            raise ValueError(f"angles need {sweep.n_angles} columns")
        self.lr, self.b1, self.b2, self.eps = float(step_size), float(b1), float(b2), float(eps)
        self.m = torch.zeros_like(self.angles)
        self.v = torch.zeros_like(self.angles)
        self.state = torch.zeros(3, dtype=torch.float64, device=dev)
        self.loss = torch.zeros(V, dtype=torch.float64, device=dev)
        self.grad = torch.zeros((V, A), dtype=torch.float64, device=dev)
        self.status = torch.zeros(V * self.inputs.shape[0], dtype=torch.int32, device=dev)
        self.losses = torch.zeros((0, V), dtype=torch.float64, device=dev)
        self._graph = None
        _native.check(_native.lib().mbqc_adam_state_init(_ptr(self.state), self.b1, self.b2, _stream_ptr(None)))

    def _iteration(self, stream=None):
        self.sweep.fidelity_grad(self.angles, self.inputs, self.targets, status=self.status, stream=stream,
                                 loss=self.loss, grad=self.grad)
        # loss row of this iteration (index from the device counter)
        idx = self.state[0:1].to(torch.int64)
        self.losses.index_copy_(0, idx, self.loss.unsqueeze(0))
        _native.check(_native.lib().mbqc_adam_step(self.angles.numel(), _ptr(self.angles), _ptr(self.grad),
                                                   _ptr(self.m), _ptr(self.v), _ptr(self.state), self.lr,
                                                   self.b1, self.b2, self.eps, _stream_ptr(stream)))

    def run(self, n_iters: int, *, graph: bool = True) -> torch.Tensor:
        """Run ``n_iters`` more iterations (asynchronously on the current
        stream); returns ``angles``."""
        done = int(self.state[0].item())
        need = done + n_iters
        if self.losses.shape[0] < need:
            grown = torch.zeros((need, self.losses.shape[1]), dtype=torch.float64, device=self.angles.device)
            grown[: self.losses.shape[0]] = self.losses
            self.losses = grown
            self._graph = None  # recorded against the old buffer
        if not graph:
            for _ in range(n_iters):
                self._iteration()
            return self.angles
        if self._graph is None and n_iters > 0:
            # the first iteration runs eagerly (warm-up, lazy allocations), the
            # rest replay one recorded iteration
            self._iteration()
            n_iters -= 1
            torch.cuda.synchronize(self.angles.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):  # records only; nothing runs during capture
                self._iteration()
            self._graph = g
        for _ in range(n_iters):
            self._graph.replay()
        return self.angles
