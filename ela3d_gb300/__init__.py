"""ela3d_gb300 -- GB300-native SEISMIC_CPML 3-D elastic C-PML time loop.

The compute runs in libela3d.so (hand-written sm_103a CUDA behind the C ABI
of include/ela3d.h); this package is the Python host mirror of that ABI plus
the workload generators.  Importing it does not load the library;
``Plan(...)`` does, and raises if the library is missing (there is no CPU
path).
"""
from ._abi import Batch, Ela3dError, ModelSpec, Plan, Server, generate_model, PlanInfo, Tuning, VariantInfo, autotune, builtin_tuning, load_library, pinned_copy, pinned_empty, select_device, variants
from .params import (FIELD_NAMES, FP32, FP64, PML_CLEAN, PML_COMPAT, SRC_EXPLOSIVE, SRC_FORCE,
                     STF_GAUSS, STF_GAUSS_DERIV, STF_RICKER, SXX, SXY, SXZ, SYY, SYZ, SZZ, VX, VY, VZ,
                     CParams, ShotParams, reference_defaults)

__all__ = [
    "Batch", "Ela3dError", "ModelSpec", "Plan", "Server", "generate_model", "PlanInfo", "Tuning", "VariantInfo", "autotune", "builtin_tuning", "load_library", "pinned_copy", "pinned_empty", "select_device", "variants", "ShotParams", "CParams", "reference_defaults",
    "FP32", "FP64", "PML_COMPAT", "PML_CLEAN", "STF_RICKER", "STF_GAUSS_DERIV", "STF_GAUSS",
    "SRC_FORCE", "SRC_EXPLOSIVE", "VX", "VY", "VZ", "SXX", "SYY", "SZZ", "SXY", "SXZ", "SYZ", "FIELD_NAMES",
]
