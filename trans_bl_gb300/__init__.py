"""GB300-native per-RK4-stage hot path of the trans_bl boundary-layer DNS.

The compute runs in the CUDA library libtransbl.so (C ABI in
include/transbl.h); this package holds its build script and a ctypes
binding.  See trans_bl_gb300.api for the Python mirror of the C ABI and
trans_bl_gb300.configs for the benchmark workloads.
"""
from . import api  # noqa: F401
