"""valomc_gb300 -- GB300-native (sm_103a) photon-packet propagation for ValoMC meshes.

The product is the native library valomc_gb300/_build/libvalomc_gb300.so (C ABI in
include/valomc_gb300.h) and the drop-in executables MC2D / MC3D beside it.  This package
holds the build recipe, a ctypes binding of the ABI (``api``) and the synthetic workloads
(``meshgen``).
"""
from . import meshgen  # noqa: F401
from .api import (VMC_FP32, VMC_FP64, Mesh, Server, VmcError, autotune, bench_fp64, bench_gather,  # noqa: F401
                  build_neighbourhood, lib, options, run, run_batch)

__all__ = ["meshgen", "run", "run_batch", "Mesh", "Server", "autotune", "options", "lib", "VmcError",
           "VMC_FP32", "VMC_FP64", "build_neighbourhood", "bench_gather", "bench_fp64"]
