"""GB300-native 3D smoke step: hand-written sm_103a CUDA kernels behind the
reference's C entry points (ZQ_CUDA_Advection3D / AddForce3D / Attenuation3D /
MACtoRegular / red-black SOR projection) and a handle-based C ABI.

The compute lives in lib/libzqs_gb300.so (built by build.py); this package is
its ctypes binding plus seeded workload builders.  Importing it does not load
the library; capi.load() does and raises when the library is missing.
"""
from . import capi, workloads  # noqa: F401

__all__ = ["capi", "workloads"]
