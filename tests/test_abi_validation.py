"""Argument checks of the C ABI that run before any device call: a NULL plan,
batch or call handle, negative batches and bad sizes come back as
MBQC_E_INVALID with a message from mbqc_last_error (no GPU needed)."""
import ctypes

import pytest

from mentpy_gb300 import _native

# entry points whose first argument is the plan
PLAN_FIRST = [
    "mbqc_sv_forward", "mbqc_sv_forward_f64", "mbqc_sv_adjoint_workspace", "mbqc_sv_adjoint",
    "mbqc_sv_adjoint_f64", "mbqc_sv_fidelity_grad", "mbqc_sv_adjoint_noalloc", "mbqc_dm_forward",
    "mbqc_dm_forward_ex", "mbqc_dm_forward_workspace", "mbqc_dm_forward_ws", "mbqc_sv_forward_sampled",
    "mbqc_sv_call_create", "mbqc_sv_sampled_workspace", "mbqc_sv_stream_workspace", "mbqc_sv_forward_stream",
    "mbqc_dm_adjoint_workspace", "mbqc_dm_adjoint", "mbqc_dm_batch_create_ex", "mbqc_dm_batch_create",
]


@pytest.fixture(scope="module")
def lib():
    from mentpy_gb300 import build

    build.build()
    return _native.lib()


def _args(fn, overrides=None):
    """One argument per parameter: NULL pointers, batch-like integers 1, zero
    doubles; output pointers (size_t / handle) point at real storage."""
    out, keep = [], []
    for i, t in enumerate(fn.argtypes):
        if overrides and i in overrides:
            out.append(overrides[i])
        elif t is ctypes.c_void_p:
            out.append(None)
        elif t in (ctypes.c_double,):
            out.append(0.0)
        elif t in (ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t):
            out.append(1)
        elif hasattr(t, "_type_"):  # a POINTER(...) type: storage it may write
            v = t._type_()
            keep.append(v)
            out.append(ctypes.pointer(v))
        else:
            raise TypeError(f"{t} in {fn.__name__}")
    return out, keep


@pytest.mark.parametrize("name", PLAN_FIRST)
def test_null_plan_is_invalid(lib, name):
    fn = getattr(lib, name)
    args, _keep = _args(fn)
    rc = fn(*args)
    assert rc == _native.MBQC_E_INVALID, (name, rc, lib.mbqc_last_error())
    assert lib.mbqc_last_error(), name


def test_null_handles_are_invalid(lib):
    for name in ("mbqc_sv_call_launch", "mbqc_dm_batch_info", "mbqc_dm_batch_forward"):
        fn = getattr(lib, name)
        args, _keep = _args(fn)
        assert fn(*args) == _native.MBQC_E_INVALID, name
    lib.mbqc_sv_call_destroy(None)  # destroying NULL is a no-op


def test_outer_rejects_bad_sizes(lib):
    for batch, n in ((-1, 2), (1, -1), (1, 16)):
        assert lib.mbqc_outer(batch, n, None, None, None) == _native.MBQC_E_INVALID
    assert b"outer" in lib.mbqc_last_error()
    assert lib.mbqc_outer(0, 3, None, None, None) == _native.MBQC_OK  # empty batch: nothing to do


def test_check_raises_with_the_library_message(lib):
    rc = lib.mbqc_sv_forward(*_args(lib.mbqc_sv_forward)[0])
    with pytest.raises(_native.MbqcError) as e:
        _native.check(rc)
    assert e.value.code == _native.MBQC_E_INVALID and str(e.value).startswith("libmbqc_gb300 error -1:")
