"""Host logic of run_batch's bound-call cache (no GPU): a buffer set is
identified by its memory, shape, strides and type, so new views of the same
memory find the bound call and other memory does not."""
import torch

from mentpy_gb300.simulators import _bind_key


def test_views_of_the_same_memory_share_a_key():
    ang = torch.zeros((4, 64, 28), dtype=torch.float64)
    out = torch.zeros((4, 64, 16), dtype=torch.complex64)
    st = torch.zeros((4, 64), dtype=torch.int32)
    k1 = _bind_key(ang[1], None, out[1], st[1], None, True, -1)
    k2 = _bind_key(ang[1], None, out[1], st[1], None, True, -1)
    assert k1 == k2 and hash(k1) == hash(k2)
    assert _bind_key(ang[2], None, out[2], st[2], None, True, -1) != k1       # other memory
    assert _bind_key(ang[1], None, out[1], st[1], None, False, -1) != k1      # other flags
    assert _bind_key(ang[1], None, out[1], st[1], None, True, 3) != k1        # other variant
    assert _bind_key(ang[1].view(torch.int64), None, out[1], st[1], None, True, -1) != k1  # other type
    assert _bind_key(ang[1][:32], None, out[1], st[1], None, True, -1) != k1  # other shape


def test_release_buffers_drops_bound_sets_after_a_device_wait(monkeypatch):
    """release_buffers waits for the device (a call in flight may still use
    the buffers) and then drops every bound set; with none bound it does not
    touch the device."""
    import types

    from mentpy_gb300.simulators import CudaSimulatorSV

    waits = []
    monkeypatch.setattr(torch.cuda, "synchronize", lambda device=None: waits.append(device))
    sim = object.__new__(CudaSimulatorSV)
    sim._sweep = types.SimpleNamespace(device="cuda:0")
    sim.release_buffers()
    assert waits == []
    sim._fast = {("k",): object()}
    sim._prepared = {("m",): object()}
    sim.release_buffers()
    assert waits == ["cuda:0"]
    assert "_fast" not in sim.__dict__ and "_prepared" not in sim.__dict__
