"""GB300-native (sm_103a) look-up-table precompute for fuzzyblue-style
precomputed atmospheric scattering.

The public API mirrors the crate's (src/lib.rs:9): Builder, Atmosphere,
Parameters, PendingAtmosphere; the compute path is libfuzzyblue_cuda.so (C ABI
in include/fuzzyblue.h).
"""
from .params import (DensityProfile, DensityProfileLayer, Parameters, PRECISION_MIXED, PRECISION_PLAIN,
                     STORAGE_F16, STORAGE_F32, dump_parameters, smoke_parameters)

__all__ = [
    "Atmosphere", "Builder", "Parameters", "PendingAtmosphere", "DensityProfile", "DensityProfileLayer",
    "build_batch", "smoke_parameters", "dump_parameters", "PRECISION_PLAIN", "PRECISION_MIXED",
    "STORAGE_F32", "STORAGE_F16",
]


def __getattr__(name):
    # The API objects need the native library; import them lazily so that
    # parameter handling works without it.
    if name in ("Atmosphere", "Builder", "PendingAtmosphere", "Server", "build_batch", "DeviceArray", "validate",
                "device_bytes"):
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
