"""The package-level names the README and INTEGRATION examples use."""


def test_readme_imports():
    import mentpy_gb300 as m
    from mentpy_gb300 import DensityMatrixSweep, PatternSimulator, StatevectorSweep  # noqa: F401

    assert PatternSimulator is m.simulators.PatternSimulator
    assert StatevectorSweep.__module__ == "mentpy_gb300.sweep"
    assert set(m.__all__) >= {"PatternSimulator", "StatevectorSweep", "DensityMatrixSweep", "many_wires"}
