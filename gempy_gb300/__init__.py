"""GB300-native co-kriging hot path of GemPy: kriging-matrix build, dense
solve, scalar-field/gradient evaluation on regular and octree grids and
sigmoid segmentation, as hand-written sm_103a CUDA kernels behind the C ABI of
``include/gempy_gb300.h``.  ``compute_model`` is a drop-in for the engine call
at ``gempy/API/compute_API.py:68-73``."""
from .data import (DEFAULT_ORI_NUGGET, DEFAULT_SP_NUGGET, CenteredGrid, EngineGrid, EvaluationOptions,
                   GenericGrid, GeophysicsInput,
                   InputDataDescriptor, InterpolationInput, InterpolationOptions, KernelFunction, KernelOptions,
                   Orientations, RegularGrid, Solutions, StackRelationType, StacksStructure, SurfacePoints,
                   TensorsStructure)
from .engine import EngineConfig, compute_model
from .transforms import Transform

__all__ = [
    "compute_model", "EngineConfig", "Transform", "InterpolationInput", "InterpolationOptions", "KernelOptions",
    "EvaluationOptions", "KernelFunction", "SurfacePoints", "Orientations", "EngineGrid", "RegularGrid",
    "GenericGrid", "InputDataDescriptor", "TensorsStructure", "StacksStructure", "StackRelationType", "Solutions",
    "DEFAULT_SP_NUGGET", "DEFAULT_ORI_NUGGET", "CenteredGrid", "GeophysicsInput",
]
