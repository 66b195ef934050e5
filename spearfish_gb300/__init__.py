"""spearfish_gb300: GB300 (sm_103a) alignment stage for spearfish's long-read mapper.

Myers bit-parallel edit distance and banded affine (Gotoh) alignment, with traceback and
CIGARs, behind the C ABI in include/sf_align.h.  ``align`` mirrors the reference's
``map::align`` entry points; ``batch`` runs thousands of jobs per launch; ``serve`` is the
serving loop (continuous batching: a host dispatcher admits requests into slots by free
HBM, and their kernels overlap on the device).
"""
from . import align, batch  # noqa: F401
from .align import Affine, Mode  # noqa: F401

__all__ = ["align", "batch", "Affine", "Mode"]
