"""incflo_gb300: GB300-native projection hot path of incflo (nodal + MAC multigrid Poisson solves).

The compute path is the CUDA library libincflo_gb300.so behind the C ABI of
include/incflo_gb300.h; this package holds its build recipe, its ctypes binding and a Python
mirror of the reference's projector interface. Nothing here computes on the CPU.
"""
from .projection import (AmrNodalProjector, Geometry, LPInfo, MacProjector, NodalProjector,  # noqa: F401
                         apply_cc_projection, apply_nodal_projection, apply_nodal_projection_boxes, array4,
                         make_options, options_from_inputs)
from ._abi import ProjectionError, load  # noqa: F401

__all__ = ["Geometry", "LPInfo", "NodalProjector", "MacProjector", "AmrNodalProjector", "apply_nodal_projection",
           "apply_nodal_projection_boxes", "apply_cc_projection",
           "array4",
           "make_options", "options_from_inputs", "ProjectionError", "load"]
