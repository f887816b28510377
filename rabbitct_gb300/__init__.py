"""rabbitct_gb300 — LolaCUDA, a GB300-native backprojection module for RabbitCT.

The product is liblolacuda.so (CUDA kernels for sm_103a + C host code) with
the C ABI in include/lolaCuda.h.  This package holds its sources (csrc/), the
in-tree build, ctypes bindings and host-side helpers that mirror the
reference's data formats and driver loop.
"""
from . import build  # noqa: F401

__all__ = ["build"]
