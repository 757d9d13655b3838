"""GB300-native non-Cartesian CG-SENSE (the NFFT / NCSENSE / CGSENSE path of codeare).

The compute path is libcgs.so (hand-written sm_103a CUDA behind the C ABI in
include/cgs.h); `capi` binds it.  There is no CPU fallback: using an operator
without the built library raises.
"""
from . import capi, synth  # noqa: F401
from .capi import Plan, CS, CgsError, MODE_CODEARE, MODE_STANDARD, kernel_launches  # noqa: F401

__all__ = ["capi", "synth", "Plan", "CS", "CgsError", "MODE_CODEARE", "MODE_STANDARD", "kernel_launches"]
