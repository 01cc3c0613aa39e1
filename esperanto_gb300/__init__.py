"""GB300-native implementation of the ESPERANTO read-alignment inner loop.

The hot path of crates/map -- the banded affine-gap Gotoh DP with traceback
to CIGAR, the editing-aware Myers filters and the splice-rescue flank DP --
runs as hand-written CUDA kernels for sm_103a behind a C ABI
(include/esperanto_gb300.h).  This package is the host-side mirror of the
reference's interface for that path (same names and semantics) plus the
batch-submit API; it has no CPU implementation of the path.
"""
from .extend import (INITIAL_BAND, DiagHint, EditDir, ExtendBuffer, ExtendParams, Extension,
                     TouchRec, extend, extend_hint, run_band)
from ._native import EspError, NativeUnavailable

__all__ = ["INITIAL_BAND", "DiagHint", "EditDir", "ExtendBuffer", "ExtendParams", "Extension",
           "TouchRec", "extend", "extend_hint", "run_band", "EspError", "NativeUnavailable"]
