"""The kernels' float reduction of double angles (``reduce_angle`` in
csrc/common.cuh), restated in numpy float32 arithmetic: its error must not
grow with |theta| (the reference takes double angles of any size,
np_simulator_sv.py:246-249, ment.py:231-232)."""
import numpy as np

F = np.float32


def _fmaf(a, b, c):
    # a*b is exact in float64 for float32 operands; one more rounding to float32
    return F(np.float64(a) * np.float64(b) + np.float64(c))


def _split2(theta):
    """t0 = top 24 significand bits (truncated), t1 = the rest rounded."""
    b = np.float64(theta).view(np.uint64)
    t0 = (b & np.uint64(0xFFFFFFFFE0000000)).view(np.float64)  # clear 29 low bits: exact truncation
    return F(t0), F(np.float64(theta) - t0)


def reduce_angle(theta):
    """Returns (r, exact_path)."""
    if abs(theta) >= 2.0**22:
        return None, True
    t0, t1 = _split2(theta)
    inv2pi = F(0.15915494309189535)
    c1 = F(6.28318548202514648)
    c2 = F(-1.7484555314695172e-07)
    k = F(np.rint(F(t0 * inv2pi)))
    r = _fmaf(-k, c1, t0)
    r = _fmaf(-k, c2, r)
    r = F(r + t1)
    if abs(r) > F(3.1415920):
        return None, True
    return r, False


def _exact(theta):
    return float(np.remainder(np.float64(theta) + np.pi, 2 * np.pi) - np.pi)


def _check(thetas, tol):
    worst, n_exact = 0.0, 0
    for th in thetas:
        r, ex = reduce_angle(th)
        if ex:
            n_exact += 1
            continue
        # compare on the circle: the double remainder itself rounds at ulp(theta)
        d = np.angle(np.exp(1j * (float(r) - _exact(th))))
        ref_err = np.spacing(abs(th))  # the double reference's own rounding
        worst = max(worst, abs(d) - ref_err)
    assert worst < tol, worst
    return n_exact


def test_small_angles():
    rng = np.random.default_rng(1)
    n = _check(rng.uniform(0, 2 * np.pi, 4000), 3e-7)
    assert n <= 2


def test_large_angles_keep_float_accuracy():
    rng = np.random.default_rng(2)
    # the float-rounded angle would be off by ulp_f32(1e4)/2 = 4.9e-4 here
    n = _check(rng.uniform(-1e4, 1e4, 4000), 3e-7)
    assert n <= 8
    n = _check(rng.uniform(-4e6, 4e6, 2000), 3e-7)
    assert n < 400  # near-half-integer quotients take the double path


def test_edge_values():
    for th in (0.0, -0.0, 1e-300, -1e-30, 1e-8, np.pi / 2, -np.pi / 2, 2 * np.pi, -2 * np.pi, 1e3 * np.pi):
        r, ex = reduce_angle(th)
        if not ex:
            assert abs(np.angle(np.exp(1j * (float(r) - _exact(th))))) < 3e-7 + np.spacing(abs(th))
    # +-pi and odd multiples go to the double path (the branch cut)
    assert reduce_angle(np.pi)[1] and reduce_angle(-3 * np.pi)[1]
    assert reduce_angle(2.0**22)[1]
