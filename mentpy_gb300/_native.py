"""ctypes binding of libmbqc_gb300.so (the C ABI declared in include/mbqc_gb300.h).

The compiled library is the only compute path: if it is missing or cannot be
loaded this module raises, there is no CPU fallback.  Build it with
``python -m mentpy_gb300.build``.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from .plan import WindowPlan

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libmbqc_gb300.so")

MBQC_OK = 0
MBQC_E_INVALID = -1
MBQC_E_CUDA = -2
MBQC_E_UNSUPPORTED = -3
MBQC_E_NOMEM = -4
MBQC_F_REF_PHASE = 1
MBQC_F_HOST_INPUTS = 2
MBQC_F_DM_EXPECTATION = 4
MBQC_F_INPUTS_READY = 8
MBQC_F_DM_FULL_MATRIX = 16
MBQC_F_STREAM_TMA = 32
RUN_OK, RUN_ZERO_NORM, RUN_NAN = 0, 1, 2

_c_int_p = ctypes.POINTER(ctypes.c_int32)
_c_u32_p = ctypes.POINTER(ctypes.c_uint32)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)


class MbqcError(RuntimeError):
    """A failed call into libmbqc_gb300 (code and the library's message)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"libmbqc_gb300 error {code}: {message}")
        self.code = code


class CircuitDesc(ctypes.Structure):
    _fields_ = [
        ("window", ctypes.c_int32),
        ("n_steps", ctypes.c_int32),
        ("n_in", ctypes.c_int32),
        ("n_out", ctypes.c_int32),
        ("n_angles", ctypes.c_int32),
        ("in_bits", _c_int_p),
        ("out_bits", _c_int_p),
        ("init_cz", _c_u32_p),
        ("step_mask", _c_u32_p),
        ("step_angle", _c_int_p),
        ("step_plane", _c_int_p),
        ("step_fixed_angle", _c_dbl_p),
    ]


class GraphDesc(ctypes.Structure):
    _fields_ = [
        ("n_nodes", ctypes.c_int32),
        ("nodes", _c_int_p),
        ("n_edges", ctypes.c_int32),
        ("edges", _c_int_p),
        ("n_inputs", ctypes.c_int32),
        ("inputs", _c_int_p),
        ("n_outputs", ctypes.c_int32),
        ("outputs", _c_int_p),
        ("plane", _c_int_p),
        ("trainable", _c_int_p),
        ("angle", _c_dbl_p),
        ("n_trainable", ctypes.c_int32),
        ("trainable_order", _c_int_p),
        ("window_size", ctypes.c_int32),
        ("kind", ctypes.c_int32),
    ]


class PlanTables(ctypes.Structure):
    _fields_ = [
        ("window", ctypes.c_int32),
        ("n_steps", ctypes.c_int32),
        ("n_in", ctypes.c_int32),
        ("n_out", ctypes.c_int32),
        ("n_angles", ctypes.c_int32),
        ("n_nodes", ctypes.c_int32),
        ("in_bits", _c_int_p),
        ("init_cz", _c_u32_p),
        ("step_mask", _c_u32_p),
        ("step_angle", _c_int_p),
        ("step_plane", _c_int_p),
        ("step_fixed_angle", _c_dbl_p),
        ("out_bits", _c_int_p),
        ("out_nodes", _c_int_p),
        ("schedule", _c_int_p),
    ]


class GraphBatchDesc(ctypes.Structure):
    _fields_ = [
        ("n_graphs", ctypes.c_int32),
        ("node_off", ctypes.POINTER(ctypes.c_int64)),
        ("nodes", _c_int_p),
        ("plane", _c_int_p),
        ("trainable", _c_int_p),
        ("angle", _c_dbl_p),
        ("edge_off", ctypes.POINTER(ctypes.c_int64)),
        ("edges", _c_int_p),
        ("in_off", ctypes.POINTER(ctypes.c_int64)),
        ("inputs", _c_int_p),
        ("out_off", ctypes.POINTER(ctypes.c_int64)),
        ("outputs", _c_int_p),
        ("window_size", ctypes.c_int32),
        ("kind", ctypes.c_int32),
    ]


class Byproducts(ctypes.Structure):
    _fields_ = [
        ("x_step", ctypes.c_void_p),
        ("z_off", ctypes.c_void_p),
        ("z_idx", ctypes.c_void_p),
        ("x_out", ctypes.c_void_p),
        ("z_out", ctypes.c_void_p),
    ]


_lib = None
_lock = threading.Lock()

_SIGS = {
    "mbqc_abi_version": (ctypes.c_int, []),
    "mbqc_last_error": (ctypes.c_char_p, []),
    "mbqc_device_sm_count": (ctypes.c_int, [_c_int_p]),
    "mbqc_compile_graph": (ctypes.c_int, [ctypes.POINTER(GraphDesc), ctypes.POINTER(PlanTables)]),
    "mbqc_adam_state_init": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "mbqc_adam_step": (ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "mbqc_plan_create_from_graphs": (ctypes.c_int, [ctypes.POINTER(GraphBatchDesc), ctypes.POINTER(ctypes.c_void_p),
                                                    ctypes.c_void_p]),
    "mbqc_mapped_pointer": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "mbqc_plan_create": (ctypes.c_int, [ctypes.POINTER(CircuitDesc), ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "mbqc_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "mbqc_sv_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32,
                                        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mbqc_sv_forward_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mbqc_sv_adjoint_workspace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                                  ctypes.POINTER(ctypes.c_size_t)]),
    "mbqc_sv_adjoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "mbqc_sv_adjoint_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "mbqc_sv_fidelity_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                              ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                              ctypes.c_void_p]),
    "mbqc_sv_adjoint_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                                ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "mbqc_dm_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    "mbqc_dm_forward_ex": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32,
                                           ctypes.c_uint64, ctypes.c_void_p]),
    "mbqc_dm_forward_workspace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                                  ctypes.POINTER(ctypes.c_size_t)]),
    "mbqc_dm_forward_ws": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32,
                                           ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "mbqc_sv_forward_sampled": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                                ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint64,
                                                ctypes.POINTER(Byproducts), ctypes.c_void_p, ctypes.c_int64,
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                ctypes.c_void_p]),
    "mbqc_sv_call_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32,
                                            ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_void_p)]),
    "mbqc_sv_call_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mbqc_sv_call_destroy": (None, [ctypes.c_void_p]),
    "mbqc_sv_sampled_workspace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    "mbqc_sv_stream_workspace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    "mbqc_sv_forward_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                               ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                               ctypes.c_void_p]),
    "mbqc_dm_adjoint_workspace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                                  ctypes.POINTER(ctypes.c_size_t)]),
    "mbqc_dm_adjoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_double, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.c_void_p]),
    "mbqc_dm_batch_create_ex": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "mbqc_dm_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                             ctypes.POINTER(ctypes.c_void_p)]),
    "mbqc_dm_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "mbqc_dm_batch_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "mbqc_dm_batch_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                              ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                              ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p]),
    "mbqc_outer": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mbqc_probe_fp32_fma": (ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                            ctypes.c_void_p]),
    "mbqc_probe_smem_bw": (ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                           ctypes.c_void_p]),
}


def exported_symbols():
    """Names of the C ABI entry points this binding expects."""
    return list(_SIGS)


def lib():
    """Load the library once; raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: the GPU backend has no fallback. "
                    "Build it with `python -m mentpy_gb300.build`."
                )
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != MBQC_OK:
        msg = lib().mbqc_last_error()
        raise MbqcError(rc, msg.decode() if msg else "")


class DevicePlan:
    """Device-resident plan table built from one or more ``WindowPlan``s."""

    @classmethod
    def from_handle(cls, handle: ctypes.c_void_p, plans) -> "DevicePlan":
        """Wrap a plan table created by the native compiler (owns it)."""
        self = cls.__new__(cls)
        self.plans = list(plans)
        self.handle = handle
        return self

    def __init__(self, plans):
        if isinstance(plans, WindowPlan):
            plans = [plans]
        self.plans = list(plans)
        keep = []
        descs = (CircuitDesc * len(self.plans))()
        for d, p in zip(descs, self.plans):
            arrs = dict(
                in_bits=np.ascontiguousarray(p.in_bits, dtype=np.int32),
                out_bits=np.ascontiguousarray(p.out_bits, dtype=np.int32),
                init_cz=np.ascontiguousarray(p.init_cz, dtype=np.uint32),
                step_mask=np.ascontiguousarray(p.step_mask, dtype=np.uint32),
                step_angle=np.ascontiguousarray(p.step_angle, dtype=np.int32),
                step_plane=np.ascontiguousarray(p.step_plane, dtype=np.int32),
                step_fixed_angle=np.ascontiguousarray(p.step_fixed_angle, dtype=np.float64),
            )
            keep.append(arrs)
            d.window, d.n_steps, d.n_in, d.n_out, d.n_angles = (
                p.window, p.n_steps, p.n_in, p.n_out, p.n_angles)
            d.in_bits = arrs["in_bits"].ctypes.data_as(_c_int_p)
            d.out_bits = arrs["out_bits"].ctypes.data_as(_c_int_p)
            d.init_cz = arrs["init_cz"].ctypes.data_as(_c_u32_p)
            d.step_mask = arrs["step_mask"].ctypes.data_as(_c_u32_p)
            d.step_angle = arrs["step_angle"].ctypes.data_as(_c_int_p)
            d.step_plane = arrs["step_plane"].ctypes.data_as(_c_int_p)
            d.step_fixed_angle = arrs["step_fixed_angle"].ctypes.data_as(_c_dbl_p)
        h = ctypes.c_void_p()
        check(lib().mbqc_plan_create(descs, len(self.plans), ctypes.byref(h)))
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib is not None:
            _lib.mbqc_plan_destroy(h)
            self.handle = None


_SMS = None


def sm_count() -> int:
    """Streaming multiprocessors of the current device."""
    global _SMS
    if _SMS is None:
        n = ctypes.c_int32()
        check(lib().mbqc_device_sm_count(ctypes.byref(n)))
        _SMS = int(n.value)
    return _SMS
