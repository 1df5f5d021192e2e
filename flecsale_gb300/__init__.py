"""flecsale_gb300: GB300-native (sm_103a) Eulerian finite-volume hydro step.

The compute path is libflecsale_gb300.so (C++ host code + hand-written CUDA
kernels behind the C ABI in include/flecsale_gb300.h).  This package exposes
that library to Python through ctypes (flecsale_gb300.hydro).
"""
from .hydro import (DeviceMesh, DeviceState, FvhError, HostMesh, Params, Solver,  # noqa: F401
                    check, initial_state, lib, make_params)

__all__ = ["DeviceMesh", "DeviceState", "FvhError", "HostMesh", "Params", "Solver",
           "check", "initial_state", "lib", "make_params"]
