"""mentpy-compatible gradient helpers (mentpy/gradients/grad.py:13-33,
_finite_difference.py:9-25, _parameter_shift.py:9-25) on plain numpy costs
(no GPU): formulas, evaluation counts and the error types the reference
raises."""
import numpy as np
import pytest

from mentpy_gb300.gradients import fd_gradient, get_gradient, psr_gradient


class Counted:
    def __init__(self, f):
        self.f, self.calls = f, 0

    def __call__(self, x):
        self.calls += 1
        return self.f(np.asarray(x))


A = np.array([[2.0, 0.5, 0.0], [0.5, 1.0, -0.3], [0.0, -0.3, 3.0]])
b = np.array([0.1, -0.2, 0.7])


def quad(x):
    return 0.5 * x @ A @ x + b @ x


def test_central_differences_are_exact_on_a_quadratic():
    x = np.array([0.3, -1.2, 2.0])
    f = Counted(quad)
    g = fd_gradient(f, x)
    assert np.allclose(g, A @ x + b, atol=1e-8)
    assert f.calls == 2 * len(x)


@pytest.mark.parametrize("kind,sign", [("forward", 1), ("backward", -1)])
def test_one_sided_differences(kind, sign):
    x = np.array([0.3, -1.2, 2.0])
    h = 1e-4
    f = Counted(quad)
    g = fd_gradient(f, x, h=h, type=kind)
    # one-sided: the gradient plus (h / 2) diag(A) in the direction of the step
    assert np.allclose(g, A @ x + b + sign * 0.5 * h * np.diag(A), atol=1e-8)
    assert f.calls == len(x) + 1


def test_parameter_shift_is_a_central_difference_with_shift_1_5():
    x = np.array([0.4, -2.0, 1.1, 3.0])
    f = Counted(lambda v: float(np.sum(np.sin(v))))
    g = psr_gradient(f, x)
    assert np.allclose(g, 2 * np.cos(x) * np.sin(1.5) / 3.0, atol=1e-12)
    assert f.calls == 2 * len(x)
    # divided by 2 * shift (not 2 sin(shift) as the textbook rule for Pauli rotations)
    assert np.allclose(psr_gradient(f, x, shift=np.pi / 2), np.cos(x) * 2 / np.pi, atol=1e-12)


def test_get_gradient_dispatch_and_errors():
    x = np.array([0.3, -1.2, 2.0])
    for m in ("parameter-shift", "psr", "parametershift"):
        assert np.allclose(get_gradient(quad, x, m), psr_gradient(quad, x))
    for m in ("finite-differences", "fd", "finitedifferences"):
        assert np.allclose(get_gradient(quad, x, m), fd_gradient(quad, x))
    assert np.allclose(get_gradient(quad, x, "fd", 1e-3, "forward"), fd_gradient(quad, x, 1e-3, "forward"))
    with pytest.raises(UserWarning, match="Expected method"):
        get_gradient(quad, x, "adjoint")
    with pytest.raises(UserWarning, match="Expected type"):
        fd_gradient(quad, x, type="sideways")


@pytest.mark.parametrize("kind", ["central", "forward", "backward"])
def test_finite_difference_hessian_of_a_quadratic(kind):
    from mentpy_gb300.gradients import fd_hessian

    x = np.array([0.3, -1.2, 2.0])
    f = Counted(quad)
    H = fd_hessian(f, x, h=1e-3, type=kind)
    assert np.allclose(H, A, atol=1e-6)
    assert f.calls == 4 * len(x) ** 2


def test_parameter_shift_hessian_and_dispatch():
    from mentpy_gb300.gradients import fd_hessian, get_hessian, psr_hessian

    x = np.array([0.4, -2.0, 1.1])
    s = 1.5
    H = psr_hessian(lambda v: float(np.sum(np.sin(v))), x)
    assert np.allclose(np.diag(H), np.sin(x) * (np.cos(2 * s) - 1) / (2 * s**2), atol=1e-12)
    assert np.allclose(H - np.diag(np.diag(H)), 0, atol=1e-12)
    for m in ("parameter-shift", "psr", "parametershift"):
        assert np.array_equal(get_hessian(quad, x, m), psr_hessian(quad, x))
    for m in ("finite-differences", "fd", "finitedifferences"):
        assert np.array_equal(get_hessian(quad, x, m), fd_hessian(quad, x))
    with pytest.raises(UserWarning, match="Expected method"):
        get_hessian(quad, x, "adjoint")
    with pytest.raises(UserWarning, match="Expected type"):
        fd_hessian(quad, x, type="sideways")


def test_helpers_give_the_references_bits():
    """Against the reference's own get_gradient / get_hessian outputs
    (tests/golden/gradients/grad_helpers.npz, made by make_golden.py
    --only-grad-helpers) on the same cost: bit for bit."""
    import os

    from mentpy_gb300.gradients import get_hessian

    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gradients",
                             "grad_helpers.npz"))
    x = z["x"]

    def cost(v):  # the fixture's cost (helper_cost in make_golden.py)
        return float(np.sin(v[0] * v[1]) + np.cos(v[2]) ** 3 + 0.37 * (v @ v) + np.exp(0.1 * v[3]))

    assert np.array_equal(get_gradient(cost, x, "parameter-shift"), z["grad_psr"])
    assert np.array_equal(get_hessian(cost, x, "parameter-shift"), z["hess_psr"])
    for t in ("central", "forward", "backward"):
        assert np.array_equal(get_gradient(cost, x, "finite-differences", 1e-4, t), z[f"grad_fd_{t}"]), t
        assert np.array_equal(get_hessian(cost, x, "finite-differences", 1e-4, t), z[f"hess_fd_{t}"]), t


def test_oracle_adam_follows_the_reference_optimizer():
    """oracle/train.py's Adam step (the device trainer's checker), fed the
    parameter-shift gradient, retraces the reference AdamOptimizer's iterates
    bit for bit (tests/golden/gradients/grad_helpers.npz)."""
    import os

    from oracle.train import adam_step

    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gradients",
                             "grad_helpers.npz"))

    def cost(v):
        return float(np.sin(v[0] * v[1]) + np.cos(v[2]) ** 3 + 0.37 * (v @ v) + np.exp(0.1 * v[3]))

    x = z["x"].copy()
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    for i, ref in enumerate(z["adam_x"]):
        x, m, v = adam_step(x, get_gradient(cost, x), m, v, i, step_size=0.1)
        assert np.array_equal(x, ref), i
