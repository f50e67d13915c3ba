"""GB300-native FDTD engine: a drop-in for Luxum's time-stepping path.

The time step runs in hand-written sm_103a CUDA kernels inside libluxum.so, reached through
the C ABI of include/luxum.h.  This package is its Python face (ctypes); the C++ command
line driver `luxum` and the C ABI are the other two.
"""
from ._ffi import (COMPONENTS, ETOTAL, EX, EY, EZ, HX, HY, HZ, LX_CPML_REFERENCE, LX_CPML_STANDARD, LX_PREC_FP16S,
                   LX_PREC_FP32, LX_PREC_FP64, LX_SRC_CW_HARD, LX_SRC_PULSE_SOFT, LuxumError, Params)
from .server import Server
from .sim import (Batch, Sim, device_bytes, field_shape, hdf5_read, hdf5_write, params, read_yaml, step_bytes,
                  trim_device_memory)

__all__ = ["Batch", "Server", "Sim", "device_bytes", "step_bytes", "field_shape", "params", "read_yaml", "hdf5_read", "hdf5_write", "Params", "LuxumError", "COMPONENTS", "EX", "EY", "EZ", "HX", "HY", "HZ",
           "ETOTAL", "LX_PREC_FP64", "LX_PREC_FP32", "LX_PREC_FP16S", "LX_CPML_REFERENCE", "LX_CPML_STANDARD",
           "LX_SRC_CW_HARD", "LX_SRC_PULSE_SOFT"]
