"""sarsolver_gb300 -- GB300 (sm_103a) implementation of sarsolver's SAR operator pair.

Public API (drop-in names of the reference where one exists):
  NumpySimpleSarOperator / GpuSarOperator   scipy LinearOperator (src/sarsolver/numpy/operator.py)
  GpuCilSarOperator / CpuSarOperator        CIL LinearOperator (src/sarsolver/cil/operator.py)
  GridSarScene, SimpleSarScene, NumpySimpleSarAperture, NumpySimpleSarDataset
  SarPlan                                   device-tensor plan under both
  cxx_binding                               single_/multi_{forward,adjoint}_evaluate
  autodiff                                  autograd Functions, phase-error gradient, autofocus
  resample                                  SRP moves and dataset downsampling on the GPU
"""
from .geometry import GridSarScene, NumpySimpleSarAperture, NumpySimpleSarDataset, SimpleSarScene, grid_axes
from .plan import SarPlan
from .operator import GpuSarOperator, NumpySimpleSarOperator
from .autodiff import (PhaseErrorSharpness, SarBackprojectFunction, SarForwardFunction, sar_backproject,
                       sar_forward, sharpness_autofocus, sharpness_gradient)

__all__ = [
    "GridSarScene", "SimpleSarScene", "NumpySimpleSarAperture", "NumpySimpleSarDataset", "grid_axes",
    "SarPlan", "NumpySimpleSarOperator", "GpuSarOperator",
    "SarForwardFunction", "SarBackprojectFunction", "sar_forward", "sar_backproject",
    "PhaseErrorSharpness", "sharpness_gradient", "sharpness_autofocus",
]
