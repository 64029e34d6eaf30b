"""GB300-native backend for mentpy's windowed MBQC measurement sweep."""
from . import circuit, plan
from .circuit import (GraphState, MBQCircuit, Ment, Measurement, find_cflow, grid_cluster, hstack,
                      linear_cluster, many_wires, muta)
from .plan import WindowPlan, compile_plan

templates = circuit
__all__ = ["GraphState", "MBQCircuit", "Ment", "Measurement", "find_cflow", "grid_cluster",
           "hstack", "linear_cluster", "many_wires", "muta", "WindowPlan", "compile_plan"]
