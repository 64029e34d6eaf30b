"""Restated optimizer of the reference, for checking the device trainer.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__``).
"""
from __future__ import annotations

import numpy as np


def adam_step(x, g, m, v, i, step_size=0.1, b1=0.9, b2=0.999, eps=1e-8):
    """One step of mentpy's AdamOptimizer.step (optimizers/adam.py:54-66) with
    the gradient ``g`` given: returns ``(x, m, v)``."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g**2
    m_hat = m / (1 - b1 ** (i + 1))
    v_hat = v / (1 - b2 ** (i + 1))
    return x - step_size * m_hat / (np.sqrt(v_hat) + eps), m, v
