"""dtrt_gb300: a GB300-native differentiable volumetric path tracer.

The product is libdtrt_gb300.so (CUDA kernels for sm_103a behind the C ABI in
include/dtrt_gb300.h). Python entry points:
  dtrt_gb300.dtrt     drop-in for the reference's native module `dtrt`
  dtrt_gb300.pydtrt   drop-in for the reference's `pydtrt` package
  dtrt_gb300.native   direct handle over the C ABI (NativeScene)
  dtrt_gb300.scenes   seeded synthetic benchmark scenes and VOL grid I/O
"""
import sys


def install_reference_names():
    """Register `dtrt` and `pydtrt` in sys.modules so reference scripts run unmodified."""
    from . import dtrt, pydtrt
    sys.modules["dtrt"] = dtrt
    sys.modules["pydtrt"] = pydtrt
    return dtrt, pydtrt
