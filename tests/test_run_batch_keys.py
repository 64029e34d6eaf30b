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
