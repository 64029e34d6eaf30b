"""Generate golden fixtures by running the reference simulators (mentpy 0.1.0a9).

Run in a container where the reference source tree is available:

    python tests/golden/make_golden.py /path/to/mentpy/checkout [--only-zexp | --only-large-angles |
                                                                  --only-grad-helpers]

mentpy imports pennylane, galois and matplotlib at module level; none of them
is on the numpy simulation path, so empty stand-in modules are registered for
them before the import.  Each case is stored as ``tests/golden/<name>.npz``:

* ``spec``        JSON: graph node order and edges, input/output nodes, the
                  measurement dict (insertion order, plane, angle), simulator
                  kwargs, and the reference's own bookkeeping
                  (``measurement_order``, ``trainable_nodes``,
                  ``quantum_output_nodes``) for checking the circuit model;
* ``angles``      float64 [R, A];
* ``inputs``      complex128 [R, 2^n_in] (absent: the default |+>^n_in);
* ``sv_state``    complex128 [R, 2^n_out]: ``run(angles, output_form="sv")``;
* ``sv_outcomes`` int [R, len(sv_outcome_nodes)];
* ``dm_rho``      complex128 [R, d, d]: numpy-dm ``run(angles)``;
* ``dm_outcomes`` int [R, len(dm_outcome_nodes)];
* ``errors``      JSON: exception type and message for invalid calls.

Inputs are generated here with a seeded generator (Haar: QR of a complex
Gaussian with the phase fix), so fixtures do not depend on mentpy's global
``np.random`` state.
"""
from __future__ import annotations

import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(root):
    for name in ("pennylane", "galois", "matplotlib", "matplotlib.pyplot",
                 "matplotlib.colors", "pathos", "pathos.multiprocessing"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["galois"].GF = lambda *a, **k: None
    sys.path.insert(0, root)
    import mentpy  # noqa: E402

    return mentpy


def haar_states(rng, n_qubits, count):
    d = 2**n_qubits
    out = np.empty((count, d), dtype=complex)
    for i in range(count):
        z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2)
        q, r = np.linalg.qr(z)
        q = q * (np.diag(r) / np.abs(np.diag(r)))
        out[i] = q[:, 0]
    return out


def circuit_spec(circ):
    g = circ.graph
    meas = []
    for node, m in circ.measurements.items():
        if m is None:
            meas.append([int(node), None, None])
        else:
            ang = m.angle
            meas.append([int(node), m.plane, None if ang is None else float(ang)])
    return {
        "nodes": [int(n) for n in g.nodes()],
        "edges": [[int(a), int(b)] for a, b in g.edges()],
        "input_nodes": [int(i) for i in circ.input_nodes],
        "output_nodes": [int(i) for i in circ.output_nodes],
        "measurements": meas,
        "measurement_order": None if circ.measurement_order is None else [int(i) for i in circ.measurement_order],
        "trainable_nodes": [int(i) for i in circ.trainable_nodes],
        "quantum_output_nodes": [int(i) for i in circ.quantum_output_nodes],
    }


def run_case(mp, name, circ, sim_kwargs, angles, inputs, kinds=("sv", "dm")):
    spec = circuit_spec(circ)
    spec["sim_kwargs"] = sim_kwargs
    data = {"angles": np.asarray(angles, dtype=float)}
    if inputs is not None:
        data["inputs"] = np.asarray(inputs, dtype=complex)
    errors = {}
    for kind in kinds:
        backend = "numpy-" + kind
        try:
            ps = mp.PatternSimulator(circ, backend=backend, **sim_kwargs)
        except Exception as exc:  # record constructor errors
            errors[kind] = [type(exc).__name__, str(exc)]
            continue
        states, outs = [], []
        for r in range(len(angles)):
            try:
                if inputs is not None:
                    ps.reset(input_state=inputs[r])
                else:
                    ps.reset()
                with np.errstate(all="ignore"):
                    if kind == "sv":
                        st = ps.run(angles[r], output_form="sv")
                    else:
                        st = ps.run(angles[r])
                states.append(np.asarray(st, dtype=complex))
                outs.append([int(v) for v in ps.outcomes.values()])
                spec[kind + "_outcome_nodes"] = [int(k) for k in ps.outcomes.keys()]
            except Exception as exc:
                errors[f"{kind}_run{r}"] = [type(exc).__name__, str(exc)]
                states.append(None)
                outs.append(None)
        if all(s is not None for s in states):
            key = "sv_state" if kind == "sv" else "dm_rho"
            data[key] = np.stack(states)
            data[kind + "_outcomes"] = np.array(outs, dtype=np.int64)
    spec["errors"] = errors
    np.savez_compressed(os.path.join(HERE, name + ".npz"), spec=json.dumps(spec), **data)
    print(f"{name}: N={len(spec['nodes'])} A={len(spec['trainable_nodes'])} "
          f"runs={len(angles)} errors={list(errors)}")


def main(root):
    mp = import_reference(root)
    T = mp.templates
    rng = np.random.default_rng(20261203)

    def angles_for(circ, runs):
        return rng.uniform(0, 2 * np.pi, size=(runs, len(circ.trainable_nodes)))

    # the benchmark configurations, at windows the reference can run
    c = T.linear_cluster(9)
    run_case(mp, "lin9", c, {}, angles_for(c, 4), None)
    run_case(mp, "lin9_haar", c, {}, angles_for(c, 4), haar_states(rng, 1, 4))
    c = T.many_wires([8] * 4)
    run_case(mp, "mw4x8", c, {}, angles_for(c, 4), haar_states(rng, 4, 4))
    c = T.many_wires([12] * 6)
    run_case(mp, "mw6x12", c, {}, angles_for(c, 2), haar_states(rng, 6, 2))
    c = T.grid_cluster(6, 4)
    run_case(mp, "grid6x4", c, {}, angles_for(c, 2), haar_states(rng, 6, 2))

    # teleportation identity (tests/test_simulators.py:13-30)
    for i in range(1, 5):
        c = T.linear_cluster(2 * i + 1)
        run_case(mp, f"teleport_lin{2*i+1}", c, {}, np.zeros((3, 2 * i)), haar_states(rng, 1, 3))

    # random-measurement cross-checks (tests/test_simulators.py:33-64), seeded
    templ = [("grid2x{}", lambda i: T.grid_cluster(2, 3 + i)),
             ("lin{}", lambda i: T.linear_cluster(3 + i)),
             ("muta21", lambda i: T.muta(2, 1))]
    for label, build in templ:
        for i in (1, 2):
            for with_x in (False, True):
                c = build(i)
                if with_x:
                    pick = rng.choice(c.outputc, 2, replace=False)
                    c[int(pick[0])] = mp.Ment("X")
                    c[int(pick[1])] = mp.Ment("X")
                w = min(5, len(c.trainable_nodes))
                nm = label.format(3 + i) if "{}" in label else f"{label}_{i}"
                nm = f"rand_{nm}_w{w}" + ("_xx" if with_x else "")
                run_case(mp, nm, c, {"window_size": w}, angles_for(c, 2), None)

    # other windows and grids
    c = T.grid_cluster(3, 5)
    run_case(mp, "grid3x5", c, {}, angles_for(c, 3), haar_states(rng, 3, 3))
    c = T.grid_cluster(3, 4)
    run_case(mp, "grid3x4_w6", c, {"window_size": 6}, angles_for(c, 2), haar_states(rng, 3, 2))
    c = T.grid_cluster(4, 4)
    run_case(mp, "grid4x4", c, {}, angles_for(c, 2), haar_states(rng, 4, 2))
    c = T.linear_cluster(6)
    run_case(mp, "lin6_w4", c, {"window_size": 4}, angles_for(c, 2), haar_states(rng, 1, 2))

    # fixed-angle and Pauli-plane measurements
    c = T.linear_cluster(7)
    c[1] = mp.Ment("X")
    c[2] = mp.Ment("Y")
    c[4] = mp.Ment(0.7, "XY")
    run_case(mp, "lin7_fixed", c, {}, angles_for(c, 3), haar_states(rng, 1, 3))

    # density-matrix outcome bookkeeping: prob0 around the 1e-4 threshold.
    # window 1 with an explicit schedule drops the CZ to the next node, so the
    # second measured qubit is a bare |+> and prob0 = cos^2(theta/2).
    c = T.linear_cluster(4)
    ang = np.array([[0.3, np.pi, 0.0], [0.3, np.pi - 0.019, 1.1], [0.3, np.pi - 0.021, 1.1],
                    [1.0, 2.0, np.pi]])
    run_case(mp, "dm_threshold_lin4_w1", c, {"window_size": 1, "schedule": [0, 1, 2, 3]}, ang,
             None, kinds=("dm",))
    # unnormalised input: the first prob0 is scaled by |psi|^2
    c = T.linear_cluster(5)
    inp = haar_states(rng, 1, 2)
    inp[0] *= 0.005
    inp[1] *= 3.0
    run_case(mp, "dm_scaled_input_lin5", c, {}, angles_for(c, 2), inp)
    # XZ / YZ planes: accepted by numpy-dm, rejected by numpy-sv
    c = T.linear_cluster(5)
    c[1] = mp.Ment(0.4, "XZ")
    c[2] = mp.Ment("YZ")
    run_case(mp, "dm_planes_lin5", c, {}, angles_for(c, 2), haar_states(rng, 1, 2))

    # error behaviour of the constructors / run
    errs = {}
    c = T.linear_cluster(5)
    for label, fn in [
        ("angles_count", lambda: mp.PatternSimulator(c, backend="numpy-sv").run([0.1, 0.2])),
        ("force0_false", lambda: mp.PatternSimulator(c, backend="numpy-sv", force0=False)),
        ("window_too_big", lambda: mp.PatternSimulator(c, backend="numpy-sv", window_size=9)),
        ("bad_backend", lambda: mp.PatternSimulator(c, backend="numpy-xx")),
        ("input_type", lambda: mp.PatternSimulator(c, backend="numpy-sv", input_state=[1, 0])),
        ("second_run", lambda: (lambda p: (p.run([0.1] * 4), p.run([0.1] * 4)))(
            mp.PatternSimulator(c, backend="numpy-sv"))),
        ("dm_angles_count", lambda: mp.PatternSimulator(c, backend="numpy-dm").run([0.1])),
    ]:
        try:
            fn()
            errs[label] = None
        except Exception as exc:
            errs[label] = [type(exc).__name__, str(exc)]
    with open(os.path.join(HERE, "errors.json"), "w") as f:
        json.dump(errs, f, indent=1, sort_keys=True)
    print("errors:", errs)


def zexp_cases(root):
    """Z-basis measurements in the density-matrix simulator's expectation mode
    (np_simulator_dm.py:327-344): the qubit is traced out unprojected and its
    outcome entry is prob1 / (prob0 + prob1), deterministically.  Stored as
    ``dm_rho`` plus ``dm_zexp_outcomes`` (float64, one column per measured node
    in the reference's outcome-dict order); own seed, so the other fixtures do
    not change."""
    mp = import_reference(root)
    T = mp.templates
    rng = np.random.default_rng(20261204)
    cases = []
    c = T.linear_cluster(5)
    c[2] = mp.Ment("Z")
    cases.append(("dm_zexp_lin5", c, haar_states(rng, 1, 3)))
    c = T.grid_cluster(2, 4)
    c[1] = mp.Ment("Z")
    cases.append(("dm_zexp_grid2x4", c, haar_states(rng, 2, 2)))
    c = T.many_wires([4, 5])
    c[5] = mp.Ment("Z")
    c[2] = mp.Ment(0.3, "XZ")
    cases.append(("dm_zexp_mw45", c, haar_states(rng, 2, 2)))
    for name, circ, inputs in cases:
        spec = circuit_spec(circ)
        spec["sim_kwargs"] = {}
        angles = rng.uniform(0, 2 * np.pi, size=(len(inputs), len(circ.trainable_nodes)))
        ps = mp.PatternSimulator(circ, backend="numpy-dm")
        rhos, outs = [], []
        for r in range(len(inputs)):
            ps.reset(input_state=inputs[r])
            rhos.append(np.asarray(ps.run(angles[r], mode="expectation"), dtype=complex))
            outs.append([float(v) for v in ps.outcomes.values()])
            spec["dm_outcome_nodes"] = [int(k) for k in ps.outcomes.keys()]
        spec["errors"] = {}
        spec["dm_mode"] = "expectation"
        np.savez_compressed(os.path.join(HERE, name + ".npz"), spec=json.dumps(spec), angles=angles,
                            inputs=np.asarray(inputs, dtype=complex), dm_rho=np.stack(rhos),
                            dm_zexp_outcomes=np.array(outs, dtype=np.float64))
        print(f"{name}: N={len(spec['nodes'])} A={len(spec['trainable_nodes'])} runs={len(inputs)}")


def large_angle_cases(root):
    """Angles far outside [0, 2pi): mentpy takes double angles of any size
    (np_simulator_sv.py:246-249, ment.py:231-232), and training loops drift
    them out of range.  Own seed, so the other fixtures do not change."""
    mp = import_reference(root)
    T = mp.templates
    rng = np.random.default_rng(20261205)
    c = T.many_wires([8] * 4)
    ang = rng.uniform(-1e4, 1e4, size=(4, len(c.trainable_nodes)))
    run_case(mp, "mw4x8_bigang", c, {}, ang, haar_states(rng, 4, 4))
    c = T.linear_cluster(9)
    ang = -rng.uniform(0, 1e3, size=(4, len(c.trainable_nodes)))
    # exact multiples of pi/2 and 2pi, and a tiny angle (not odd multiples of
    # pi: there the projected qubit is |->, whose halves the summing partial
    # trace (state_ops.py:69) cancels to rounding noise, so the reference's
    # statevector output is not defined)
    ang[0, :3] = [-np.pi / 2, 2 * np.pi, 1e-9]
    run_case(mp, "lin9_negang", c, {}, ang, haar_states(rng, 1, 4))
    c = T.many_wires([12] * 6)
    ang = rng.uniform(-1e4, 1e4, size=(2, len(c.trainable_nodes)))
    run_case(mp, "mw6x12_bigang", c, {}, ang, haar_states(rng, 6, 2))
    c = T.grid_cluster(3, 5)
    ang = rng.uniform(-3e5, 3e5, size=(3, len(c.trainable_nodes)))
    run_case(mp, "grid3x5_hugeang", c, {}, ang, haar_states(rng, 3, 3))


def helper_cost(v):
    """A fixed smooth cost of four angles (the same expression in the test that
    reads the fixture)."""
    return float(np.sin(v[0] * v[1]) + np.cos(v[2]) ** 3 + 0.37 * (v @ v) + np.exp(0.1 * v[3]))


def gradient_helper_case(root):
    """gradients/grad_helpers.npz: the reference's get_gradient / get_hessian
    (gradients/grad.py) of helper_cost at a seeded point, every method and
    finite-difference type, and the iterates of its Adam optimizer from that
    point."""
    mp = import_reference(root)
    from mentpy.gradients import get_gradient, get_hessian

    x = np.random.default_rng(20260417).uniform(-2, 2, 4)
    out = {"x": x}
    for m in ("parameter-shift", "finite-differences"):
        key = "psr" if m == "parameter-shift" else "fd"
        if key == "psr":
            out["grad_psr"] = get_gradient(helper_cost, x, m)
            out["hess_psr"] = get_hessian(helper_cost, x, m)
            continue
        for t in ("central", "forward", "backward"):
            out[f"grad_fd_{t}"] = get_gradient(helper_cost, x, m, 1e-4, t)
            out[f"hess_fd_{t}"] = get_hessian(helper_cost, x, m, 1e-4, t)
    os.makedirs(os.path.join(HERE, "gradients"), exist_ok=True)  # apart from the circuit fixtures
    # mentpy's Adam (optimizers/adam.py:54-66) on the same cost, its default
    # parameter-shift gradient: every iterate of 20 steps
    from mentpy.optimizers import AdamOptimizer

    traj = []
    AdamOptimizer(step_size=0.1).optimize(helper_cost, x.copy(), num_iters=20,
                                          callback=lambda xi, i: traj.append(np.array(xi)))
    out["adam_x"] = np.array(traj)
    np.savez(os.path.join(HERE, "gradients", "grad_helpers.npz"), **out)
    print("grad_helpers", mp.__name__)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not args:
        sys.exit("usage: make_golden.py /path/to/mentpy/checkout "
                 "[--only-zexp | --only-large-angles | --only-grad-helpers]")
    root = args[0]
    if "--only-zexp" in sys.argv:
        zexp_cases(root)
    elif "--only-large-angles" in sys.argv:
        large_angle_cases(root)
    elif "--only-grad-helpers" in sys.argv:
        gradient_helper_case(root)
    else:
        main(root)
        zexp_cases(root)
        large_angle_cases(root)
        gradient_helper_case(root)
