"""MatrixMarket ingest on the GPU (fl_mtx_* in include/fastload.h).

Mtx.read parses a coordinate .mtx file on the device into CSR exactly as the
reference's mmio_allinone (src/auxiliary.h:64-232) reads it; Plan.from_mtx
(plan.py) builds a FastLoad plan from that device CSR without a host round
trip; mmio_allinone returns the same CSR as host arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import MtxInfoC, check, load

REAL, INTEGER, PATTERN, COMPLEX = 0, 1, 2, 3
GENERAL, SYMMETRIC, HERMITIAN, SKEW = 0, 1, 2, 3


def _stream(stream):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Mtx:
    """A .mtx file parsed into device CSR (owned by the handle)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        i = MtxInfoC()
        check(load().fl_mtx_info_get(self._h, C.byref(i)))
        self.info = {k: getattr(i, k) for k, _ in MtxInfoC._fields_}
        self.m, self.n, self.nnz = self.info["m"], self.info["n"], self.info["nnz"]

    @classmethod
    def read(cls, path, stream=None) -> "Mtx":
        h = C.c_void_p()
        check(load().fl_mtx_read(C.byref(h), str(path).encode(), _stream(stream)))
        return cls(h)

    def device_pointers(self) -> tuple[int, int, int]:
        """(row pointer, column indices, values) device addresses, valid
        while the handle lives."""
        rp, ci, v = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(load().fl_mtx_csr(self._h, C.byref(rp), C.byref(ci), C.byref(v)))
        return rp.value or 0, ci.value or 0, v.value or 0

    def to_torch(self, stream=None):
        """Copies of (rowptr int32, colidx int32, val float64) as CUDA tensors."""
        import torch

        rp = torch.empty(self.m + 1, dtype=torch.int32, device="cuda")
        ci = torch.empty(self.nnz, dtype=torch.int32, device="cuda")
        v = torch.empty(self.nnz, dtype=torch.float64, device="cuda")
        check(load().fl_mtx_copy_csr(self._h, C.c_void_p(rp.data_ptr()), C.c_void_p(ci.data_ptr() if self.nnz else 0),
                                     C.c_void_p(v.data_ptr() if self.nnz else 0), _stream(stream)))
        return rp, ci, v

    def close(self) -> None:
        if self._h:
            load().fl_mtx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def mmio_allinone(filename):
    """(m, n, nnz, isSymmetric, rowptr, colidx, val) as numpy arrays, parsed
    on the GPU (fl_mmio_allinone, the reference's mmio_allinone)."""
    m, n, nnz, sym = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    rp, ci = C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    v = C.POINTER(C.c_double)()
    lib = load()
    check(lib.fl_mmio_allinone(C.byref(m), C.byref(n), C.byref(nnz), C.byref(sym), C.byref(rp), C.byref(ci),
                               C.byref(v), str(filename).encode()))
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    try:
        rowptr = np.ctypeslib.as_array(rp, (m.value + 1,)).copy()
        colidx = np.ctypeslib.as_array(ci, (max(nnz.value, 1),))[:nnz.value].copy()
        val = np.ctypeslib.as_array(v, (max(nnz.value, 1),))[:nnz.value].copy()
    finally:
        for ptr in (rp, ci, v):
            libc.free(C.cast(ptr, C.c_void_p))
    return m.value, n.value, nnz.value, sym.value, rowptr, colidx, val
