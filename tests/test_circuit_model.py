"""The host circuit model reproduces the reference's bookkeeping exactly:
measurement order, trainable-node order (the angle-vector layout) and quantum
outputs, checked against the reference's own values stored in the fixtures."""
import numpy as np
import pytest

from helpers import circuit_from_spec, golden_names, load_golden
from mentpy_gb300 import circuit as C


@pytest.mark.parametrize("name", golden_names())
def test_bookkeeping_matches_reference(name):
    spec, _ = load_golden(name)
    circ = circuit_from_spec(spec)
    assert list(circ.graph.nodes()) == spec["nodes"]
    assert circ.measurement_order == spec["measurement_order"]
    assert circ.trainable_nodes == spec["trainable_nodes"]
    assert circ.quantum_output_nodes == spec["quantum_output_nodes"]


@pytest.mark.parametrize(
    "name,build",
    [
        ("lin9", lambda: C.linear_cluster(9)),
        ("mw4x8", lambda: C.many_wires([8] * 4)),
        ("mw6x12", lambda: C.many_wires([12] * 6)),
        ("grid6x4", lambda: C.grid_cluster(6, 4)),
        ("grid3x5", lambda: C.grid_cluster(3, 5)),
        ("rand_muta21_1_w5", lambda: C.muta(2, 1)),
    ],
)
def test_templates_match_reference(name, build):
    spec, _ = load_golden(name)
    circ = build()
    assert list(circ.graph.nodes()) == spec["nodes"]
    assert sorted(map(sorted, circ.graph.edges())) == sorted(map(sorted, spec["edges"]))
    assert circ.input_nodes == spec["input_nodes"]
    assert circ.output_nodes == spec["output_nodes"]
    assert circ.measurement_order == spec["measurement_order"]
    assert circ.trainable_nodes == spec["trainable_nodes"]


def test_large_template_orders():
    # column-major order across wires/rows (verified on the reference)
    mw = C.many_wires([8] * 4)
    assert mw.measurement_order[:8] == [0, 8, 16, 24, 1, 9, 17, 25]
    g = C.grid_cluster(16, 10)
    assert g.measurement_order[:17] == [10 * r for r in range(16)] + [1]
    assert len(g.trainable_nodes) == 144


def test_ment_rules():
    assert C.Ment("X").angle == 0 and not C.Ment("X").is_trainable()
    assert C.Ment().is_trainable()
    assert C.Ment(0.5, "XY").angle == 0.5
    with pytest.raises(ValueError):
        C.Ment(0.3, "Z")
    with pytest.raises(ValueError):
        C.Ment(plane="QQ")
    p0, p1 = C.Ment("XY").get_povm(0.7)
    assert np.allclose(p0 + p1, np.eye(2))
    assert np.allclose(p0 @ p0, p0)
