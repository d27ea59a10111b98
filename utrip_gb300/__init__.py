"""GB300 (sm_103a) implementation of the CANS ideal-MHD modified Lax-Wendroff
step, reached through the C ABI of libcansgpu.so (include/cans_gpu.h).

`capi` binds the library with the reference routine names (mlw_m3, cfl_m3,
bd*, ...) and the device-resident run handle; `setups` builds the model
set-ups of the benchmark configurations; `drivers` reproduces the reference
model-package time loops on top of the C ABI.
"""
from . import capi, setups  # noqa: F401
from .capi import (CansError, Run, bd, cfl_m, cfl_m3, load, mlw_m, mlw_m3,  # noqa: F401
                   pull, push, register, release)

__all__ = ["capi", "setups", "CansError", "Run", "bd", "cfl_m", "cfl_m3", "load",
           "mlw_m", "mlw_m3", "pull", "push", "register", "release"]
