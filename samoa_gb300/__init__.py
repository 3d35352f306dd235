"""samoa_gb300: GB300-native (sm_103a) drop-in for sam(oa)^2's SWE explicit Euler time step.

The product boundary is the C ABI of libsamoa_swe.so (include/samoa_swe.h);
this package is its Python host side: mesh generation, scenario setup and a
mirror of the reference traversal interface.
"""
from .swe import (AUG_RIEMANN, BC_NOSLIP, BC_OUTFLOW, BC_SLIP, FWAVE, LF, LF_BATH, LLF, LLF_BATH, Config, Grid,
                  Mesh, SweContext, SweEulerTimestepTraversal, initial_dt, uniform_mesh)

__all__ = ["Config", "Grid", "Mesh", "SweContext", "SweEulerTimestepTraversal", "uniform_mesh", "initial_dt",
           "FWAVE", "AUG_RIEMANN", "LF", "LF_BATH", "LLF", "LLF_BATH", "BC_OUTFLOW", "BC_SLIP", "BC_NOSLIP"]
