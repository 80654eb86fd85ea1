"""sparsedist_gb300 -- the blocked exact-kNN path of sparseDist on GB300.

The public functions mirror the reference's R interface (see api.py); the
computation runs in libsdgpu.so (include/sdgpu.h) on the GPU.
"""
from ._lib import SdgError, Context, NA_INTEGER, NA_REAL_BITS, load as load_library  # noqa: F401
from .api import (KNNResult, SparseDistWarning, is_na, NA_REAL, sparseDist, sparseKNN,  # noqa: F401
                  sparseKNNCross, sparseSNN, snnJaccard, topKBlock, topKRowsAccum)

__all__ = ["sparseKNN", "sparseKNNCross", "sparseSNN", "sparseDist", "topKBlock",
           "topKRowsAccum", "snnJaccard", "KNNResult", "SdgError", "SparseDistWarning",
           "Context", "is_na", "NA_INTEGER", "NA_REAL", "load_library"]
