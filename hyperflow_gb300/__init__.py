"""GB300-native reacting-Euler step of HyperFlow V3 (flux, ghost fill, chemistry).

The compute path is libhyperflow_gpu.so (hand-written CUDA for sm_103a behind the
C ABI of include/hyperflow_gpu.h); this package binds it with ctypes and keeps the
reference's per-block names (see solver.py).  There is no CPU fallback.
"""
from .solver import (AmrStepper, ChemistryBatch, ChemObjective, ChemSensitivity, ConservativeInterp, Context,  # noqa
                     DomainError, FlowAdjoint, HyperFlowError, PatchArray, PatchSet, Stepper, admissible,
                     average_down, cfl_dt, euler_stage, fill, flux_adjoint, hllc, induction_length, make_level,
                     properties, reflux, repair_roundoff, tag_cells, totals, validate)

__all__ = ["AmrStepper", "ChemistryBatch", "ChemObjective", "ChemSensitivity", "ConservativeInterp", "Context", "DomainError",
           "FlowAdjoint", "HyperFlowError", "induction_length", "PatchArray", "PatchSet", "Stepper", "admissible", "average_down", "cfl_dt", "euler_stage",
           "fill", "flux_adjoint", "hllc", "make_level", "properties", "reflux", "repair_roundoff", "tag_cells", "totals",
           "validate"]
