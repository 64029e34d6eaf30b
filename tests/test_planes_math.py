"""XZ / YZ measurements in the statevector sweep (no GPU): the reference
statevector simulator rejects them (np_simulator_sv.py:53-59), its
density-matrix simulator takes them.  The kernels apply the reference's own
step -- project, sum the measured qubit out (state_ops.py:69), renormalise --
with the coefficients restated here."""
import numpy as np
import pytest

from helpers import circuit_from_spec, exec_plan_sv, haar_states, load_golden
from mentpy_gb300 import circuit as C
from mentpy_gb300.plan import compile_plan
from oracle import sweep as oracle


def coef_gen(plane, theta):
    """(amp, c, ph) of csrc/common.cuh sv_coef_gen for XZ / YZ."""
    r = np.angle(np.exp(1j * theta))  # reduced to [-pi, pi]
    C_, S_ = np.cos(r / 2), np.sin(r / 2)
    amp, d = C_ + S_, C_ - S_
    sg = -1.0 if amp < 0 else 1.0  # the sign moves from the contraction to the phase
    amp, d = sg * amp, sg * d
    if plane == "XZ":
        return amp, complex(d), sg + 0j
    return amp, -1j * d, (amp + 1j * d) / np.sqrt(2)


@pytest.mark.parametrize("plane", ["XZ", "YZ"])
def test_coefficients_are_the_reference_step(plane):
    rng = np.random.default_rng(3)
    for theta in list(rng.uniform(-50, 50, 200)) + [0.0, np.pi / 2, -np.pi / 2, 1.0]:
        p0, _ = oracle.povm(plane, theta)
        amp, c, ph = coef_gen(plane, theta)
        # the reference step: phi_ref = sum_b colsum_b psi_b with colsum = column sums of P0
        colsum = p0[0, :] + p0[1, :]
        # kernel: ph * |v0 + v1| * (amp psi0 + c psi1) / sqrt(2), v = conj((amp, c)) / sqrt(2)
        v = np.conj(np.array([amp, c])) / np.sqrt(2)
        assert np.allclose(np.outer(v, v.conj()), p0, atol=1e-12)
        # the reference's eigenvector convention, v0 = sqrt(P0[0,0]) >= 0: the
        # contraction without its phase is the reference's with the phase divided out
        assert np.isclose(v[0], np.sqrt(p0[0, 0].real), atol=1e-12)
        s = v[0] + v[1]
        if abs(s) > 1e-6:
            assert np.isclose(ph, s / abs(s), atol=1e-12)
            assert np.allclose(colsum, s * np.conj(v), atol=1e-12)


def _planes_circuit(n, planes):
    c = C.linear_cluster(n)
    for node, pl in planes.items():
        c[node] = C.Ment(pl)
    return c


@pytest.mark.parametrize("planes", [{1: "XZ"}, {2: "YZ"}, {1: "XZ", 2: "YZ", 4: "XZ"}, {0: "YZ", 3: "XZ"}])
def test_extended_plan_matches_oracle(planes):
    circ = _planes_circuit(7, planes)
    with pytest.raises(ValueError, match="only XY plane"):
        compile_plan(circ, "sv")
    plan = compile_plan(circ, "sv", extended_planes=True)
    rng = np.random.default_rng(5)
    for _ in range(4):
        ang = rng.uniform(-10, 10, size=plan.n_angles)
        psi = haar_states(rng, 1, 1)[0]
        ref, _, _ = oracle.run_sv(circ, ang, psi, output_form="sv")
        assert np.allclose(exec_plan_sv(plan, ang, psi), ref, atol=1e-10)


def test_extended_statevector_reproduces_the_reference_density_matrix():
    """The reference's numpy-dm output on its XZ / YZ fixture equals the outer
    product of the statevector sweep with those planes."""
    spec, data = load_golden("dm_planes_lin5")
    circ = circuit_from_spec(spec)
    plan = compile_plan(circ, "sv", extended_planes=True)
    for r in range(len(data["angles"])):
        sv = exec_plan_sv(plan, data["angles"][r], data["inputs"][r])
        assert np.allclose(np.outer(sv, sv.conj()), data["dm_rho"][r], atol=1e-10)


@pytest.mark.parametrize("plane", ["XZ", "YZ"])
def test_coefficient_derivatives_of_the_adjoint(plane):
    """The derivatives the block-per-run adjoint uses for XZ / YZ steps
    (csrc/sv_adj_wide.cu): XZ d amp = c / 2, dc = -amp / 2; YZ d amp =
    -Im(c) / 2, dc = i amp / 2 -- against central differences of the
    coefficients (away from the branch cut and the sign switch of amp)."""
    rng = np.random.default_rng(5)
    h = 1e-6
    for theta in rng.uniform(-np.pi + 0.01, np.pi - 0.01, 300):
        amp, c, _ = coef_gen(plane, theta)
        ap, cp, _ = coef_gen(plane, theta + h)
        am, cm, _ = coef_gen(plane, theta - h)
        if np.sign(ap) != np.sign(am) or abs(amp) < 1e-3:
            continue  # the sign moves into the phase here: piecewise
        damp_fd, dc_fd = (ap - am) / (2 * h), (cp - cm) / (2 * h)
        if plane == "XZ":
            damp, dc = 0.5 * c.real, -0.5 * amp + 0j
        else:
            damp, dc = -0.5 * c.imag, 0.5j * amp
        assert abs(damp - damp_fd) < 1e-6 and abs(dc - dc_fd) < 1e-6, theta
