"""fastload_gb300 -- GB300-native (sm_103a) FastLoad CSC SpMV engine.

Host entry points keep the reference's names (csr_to_csc, ColSort,
formatTransform, FastLoad_spmv); Plan is the device-resident API.  Every
computation runs in the CUDA library; importing the package raises
ImportError when that library is missing.
"""
from ._lib import FastLoadArgumentError, FastLoadError, load
from .batch import Batch
from .host import ColSort, FastLoad_spmv, SlideMatrix, csr_to_csc, formatTransform
from .mtx import Mtx, mmio_allinone
from .plan import (BAND_ALL, BAND_AUTO, BAND_NONE, INPUT_CSC, INPUT_CSR, KERNEL_AUTO, KERNEL_BUCKET, KERNEL_STREAM,
                   KERNEL_STREAM2, KERNEL_TILE, VALUES_BF16X2, VALUES_F32, VALUES_F64, HEAVY_AUTO, HEAVY_RING, HEAVY_REGS,
                   XSTAGE_AUTO, XSTAGE_GLOBAL, Plan, convert_values)

load()

__all__ = [
    "FastLoadError", "FastLoadArgumentError", "SlideMatrix", "Batch", "Mtx", "mmio_allinone", "csr_to_csc", "ColSort", "formatTransform", "FastLoad_spmv", "Plan",
    "KERNEL_AUTO", "KERNEL_TILE", "KERNEL_STREAM", "KERNEL_STREAM2", "KERNEL_BUCKET", "INPUT_CSR", "INPUT_CSC",
    "VALUES_F64", "VALUES_F32", "VALUES_BF16X2", "BAND_AUTO", "BAND_NONE", "BAND_ALL", "load", "convert_values",
    "HEAVY_AUTO", "HEAVY_RING", "HEAVY_REGS", "XSTAGE_AUTO", "XSTAGE_GLOBAL",
]
