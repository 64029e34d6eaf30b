"""GB300-native backend for mentpy's windowed MBQC measurement sweep."""
from . import circuit, plan
from .circuit import (GraphState, MBQCircuit, Ment, Measurement, find_cflow, grid_cluster, hstack,
                      linear_cluster, many_wires, muta)
from .plan import WindowPlan, compile_plan

templates = circuit
__all__ = ["GraphState", "MBQCircuit", "Ment", "Measurement", "find_cflow", "grid_cluster",
           "hstack", "linear_cluster", "many_wires", "muta", "WindowPlan", "compile_plan",
           "PatternSimulator", "StatevectorSweep", "DensityMatrixSweep"]

# the simulators need torch and the native library: imported on first use
_LAZY = {"PatternSimulator": "simulators", "StatevectorSweep": "sweep", "DensityMatrixSweep": "dm"}


def __getattr__(name):
    mod = _LAZY.get(name)
    if mod is None:
        raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
    import importlib

    return getattr(importlib.import_module(f".{mod}", __name__), name)
