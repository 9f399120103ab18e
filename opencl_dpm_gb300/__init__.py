"""GB300-native (sm_103a) Deformable Particle Model step.

The product is the native library ``libdpm_gb300.so`` (C ABI in
``include/dpm_gb300.h``) and the ``clDPM`` module built on it, which mirrors
the reference's Python API (Cell2D, Tissue2D, Cell3D, Tissue3D).  There is no
CPU or OpenCL fallback: importing ``clDPM`` or creating a context fails
loudly when the native library is absent.
"""
import os

__all__ = ["abi", "LIB_PATH"]
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libdpm_gb300.so")
