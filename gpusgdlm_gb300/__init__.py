"""GB300-native SGDLM online filtering (drop-in for rSGDLM's ``SGDLM`` class).

``SGDLM`` mirrors the reference's Rcpp module surface; the compute runs in the
in-tree CUDA library ``libsgdlm_gb300.so`` (hand-written sm_103a kernels behind
the C ABI of include/sgdlm.h).  There is no CPU fallback.
"""
from .sgdlm import SGDLM, Batch, SGDLMError, encode_sp, NA_UNSIGNED  # noqa: F401
from . import _lib  # noqa: F401

__all__ = ["SGDLM", "Batch", "SGDLMError", "encode_sp", "NA_UNSIGNED"]
