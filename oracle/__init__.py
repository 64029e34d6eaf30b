"""CPU oracle for the windowed MBQC sweep -- TEST INFRASTRUCTURE ONLY.

Nothing in the product package imports this directory.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of
``bench.py`` use it, and only as the checker or as the timed CPU baseline.

Modules
-------
``sweep``        complex128 restatement of mentpy's windowed statevector and
                 density-matrix sweeps, O(2^w) per step, any window size.
``dense``        the same sweep with mentpy's own dense 2^w x 2^w operators:
                 the reference algorithm, used as the timed CPU baseline.
``fullcircuit``  whole-graph density-matrix simulation with PennyLane's
                 placement of depolarising noise (every qubit once, after the
                 CZ layer); pins the windowed noise model on small graphs.
``gradients``    complex128 fidelity loss and its central finite-difference
                 gradient, the check for the adjoint kernels.
``train``        mentpy's Adam step restated, the check for the device trainer.

Parity of ``sweep`` and ``dense`` is pinned against outputs of the reference
itself (mentpy 0.1.0a9 run in the build container), committed as fixtures in
``tests/golden`` together with the script that generated them.
"""
