"""The index algebra behind the streamed kernel's table-driven first window
(csrc/sv_stream.cu, stream_init): for a chunk bit set S of the window, the
input gather x and the initial-CZ quadratic form Q split over idx = hi | lo,
and the lo tables can be built by doubling over S.  Brute force over random
CZ tables, input-bit orders and windows (no GPU)."""
import numpy as np
import pytest


def _popc(x):
    return bin(x).count("1")


def _gather(idx, bits):
    x = 0
    for b in bits:
        x = (x << 1) | ((idx >> b) & 1)
    return x


def _q(idx, cz, w):
    p = 0
    for q in range(w):
        p ^= ((idx >> q) & 1) & (_popc(idx & cz[q]) & 1)
    return p


def _chunk_bits(w, in_bits, k_max=11):
    # window bits 0..4, then the window bits of the lowest input bits, then the lowest others
    k = min(w, k_max)
    s = set(range(5))
    n_in = len(in_bits)
    for j in range(min(6, n_in)):
        if len(s) >= k:
            break
        s.add(in_bits[n_in - 1 - j])
    for b in range(w):
        if len(s) >= k:
            break
        s.add(b)
    return sorted(s)


@pytest.mark.parametrize("seed", range(20))
def test_init_tables_by_doubling(seed):
    rng = np.random.default_rng(seed)
    w = int(rng.integers(8, 21))
    cz = [int(rng.integers(0, 2**w)) for _ in range(w)]
    n_in = int(rng.integers(1, w + 1))
    in_bits = [int(b) for b in rng.permutation(w)[:n_in]]
    S = _chunk_bits(w, in_bits)
    K = len(S)
    assert S[:5] == [0, 1, 2, 3, 4]
    xt, qt = [0] * (1 << K), [0] * (1 << K)
    for b in range(K):
        pb = S[b]
        nb = 0
        for i in range(b):
            nb |= (((cz[pb] >> S[i]) ^ (cz[S[i]] >> pb)) & 1) << i
        xb, qb = _gather(1 << pb, in_bits), _q(1 << pb, cz, w)
        for l in range(1 << b):
            xt[(1 << b) | l] = xb | xt[l]
            qt[(1 << b) | l] = qb ^ qt[l] ^ (_popc(l & nb) & 1)
    smask = sum(1 << p for p in S)
    for _ in range(64):
        idx = int(rng.integers(0, 2**w))
        lo, hi = idx & smask, idx & ~smask
        l = sum(1 << i for i, p in enumerate(S) if (lo >> p) & 1)
        acc = 0
        for q in range(w):
            if (hi >> q) & 1:
                acc ^= cz[q]
        m = sum((((acc >> p) ^ _popc(hi & cz[p])) & 1) << i for i, p in enumerate(S))
        assert _q(hi, cz, w) ^ qt[l] ^ (_popc(l & m) & 1) == _q(idx, cz, w)
        assert _gather(hi, in_bits) | xt[l] == _gather(idx, in_bits)


def _mixed_passes(w, m):
    out, k = [], 0
    while k < m:
        phase, hi, lo, seq = 0, 0, 0, []
        while k < m:
            b = k % w
            if b < 5:
                if phase == 2 or lo == 5:
                    break
                phase, lo = 1, lo + 1
            else:
                if hi == 5:
                    break
                phase, hi = (2 if phase == 1 else phase), hi + 1
            seq.append(b)
            k += 1
        out.append(seq)
    return out


@pytest.mark.parametrize("w,m", [(10, 60), (11, 50), (17, 144), (19, 38), (30, 300)])
def test_mixed_pass_schedule(w, m):
    """Passes cover every step once, in order, each of the form high* low*
    high* with at most five high and five distinct low bits."""
    passes = _mixed_passes(w, m)
    assert [b for p in passes for b in p] == [k % w for k in range(m)]
    for p in passes:
        kinds = "".join("l" if b < 5 else "h" for b in p)
        assert kinds.count("h") <= 5 and kinds.count("l") <= 5
        stripped = kinds.strip("h")
        assert "h" not in stripped  # the low steps are one contiguous run
        assert len(set(p)) == len(p)
    if w == 17 and m == 144:
        assert len(passes) == 20


@pytest.mark.parametrize("seed", range(12))
def test_epilogue_chunk_tables(seed):
    """The streamed epilogue's output chunks (csrc/sv_stream.cu, make_out_desc):
    chunk-local index l enumerates the window bits of output bits 0..K-1 in
    increasing window order; its output offset and window offset agree with
    the direct output -> window map, and every output is written once."""
    rng = np.random.default_rng(100 + seed)
    w = int(rng.integers(8, 20))
    n_out = int(rng.integers(1, w + 1))
    out_bits = [int(b) for b in rng.permutation(w)[:n_out]]  # window bit of output j
    ywin = [out_bits[n_out - 1 - j] for j in range(n_out)]  # window bit of y bit j
    K = min(n_out, 10)
    order = sorted(range(K), key=lambda i: ywin[i])

    def wl(l):
        return sum(1 << ywin[order[i]] for i in range(K) if (l >> i) & 1)

    def yl(l):
        return sum(1 << order[i] for i in range(K) if (l >> i) & 1)

    def to_window(y):
        return sum(1 << ywin[j] for j in range(n_out) if (y >> j) & 1)

    assert sorted(yl(l) for l in range(1 << K)) == list(range(1 << K))
    assert all(wl(l) < wl(l + 1) for l in range((1 << K) - 1))  # window order
    seen = set()
    for ch in rng.choice(1 << (n_out - K), min(4, 1 << (n_out - K)), replace=False):
        base = to_window(int(ch) << K)
        for l in range(1 << K):
            y = (int(ch) << K) | yl(l)
            assert base | wl(l) == to_window(y)
            seen.add(y)
    assert len(seen) == len(set(seen))
