"""fastload_gb300 -- GB300-native (sm_103a) FastLoad CSC SpMV engine.

Host entry points keep the reference's names (csr_to_csc, ColSort,
formatTransform, FastLoad_spmv); Plan is the device-resident API.  Every
computation runs in the CUDA library; importing the package raises
ImportError when that library is missing.
"""
from ._lib import FastLoadError, load
from .host import ColSort, FastLoad_spmv, SlideMatrix, csr_to_csc, formatTransform
from .plan import INPUT_CSC, INPUT_CSR, KERNEL_AUTO, KERNEL_BUCKET, KERNEL_STREAM, KERNEL_STREAM2, KERNEL_TILE, Plan

load()

__all__ = [
    "FastLoadError", "SlideMatrix", "csr_to_csc", "ColSort", "formatTransform", "FastLoad_spmv", "Plan",
    "KERNEL_AUTO", "KERNEL_TILE", "KERNEL_STREAM", "KERNEL_STREAM2", "KERNEL_BUCKET", "INPUT_CSR", "INPUT_CSC",
    "load",
]
