"""GB300-native OpenPixi hot path: temporal-gauge Yang-Mills leapfrog, CPIC
(NGP) coupling and the energy / Gauss-law reductions as sm_103a kernels behind
the C ABI of ``libopixi_gpu.so`` (include/opixi.h), with a host-side mirror of
the reference's Java API (Settings, Simulation, Grid, FieldSolver,
Diagnostics, YAML input)."""
from ._native import (Handle, Batch, OpixiError, PinnedArray, OPX_F32, OPX_F64, FIELD_U, FIELD_UNEXT,
                      FIELD_E, FIELD_J, FIELD_RHO, LAYOUT_REF, LAYOUT_GEN)

__all__ = ["Handle", "Batch", "OpixiError", "PinnedArray", "OPX_F32", "OPX_F64", "FIELD_U", "FIELD_UNEXT",
           "FIELD_E", "FIELD_J", "FIELD_RHO", "LAYOUT_REF", "LAYOUT_GEN"]
