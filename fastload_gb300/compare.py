"""Comparators for reports (fl_csc_spmv_naive, fl_cusparse_* in
include/fastload.h): the reference's naive one-thread-per-column CSC kernel
and cuSPARSE CSR SpMV on device tensors, timed like the FastLoad kernels.
They give context lines in benchmarks and are never used as a fallback."""
from __future__ import annotations

import ctypes as C

from ._lib import check, load
from .plan import _need_cuda


def _torch():
    import torch

    return torch


def _stream(stream):
    s = stream if stream is not None else _torch().cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def csc_spmv_naive(m, colptr, rowidx, val, x, y=None, accumulate=False, stream=None):
    """y = A x (original column order) with the naive CSC kernel."""
    torch = _torch()
    n = colptr.numel() - 1
    _need_cuda(x, torch.float64, n, "csc_spmv_naive x")
    if y is None:
        y = torch.empty(m, dtype=torch.float64, device="cuda")
        accumulate = False
    else:
        _need_cuda(y, torch.float64, m, "csc_spmv_naive y")
    check(load().fl_csc_spmv_naive(m, n, rowidx.numel(), C.c_void_p(colptr.data_ptr()),
                                   C.c_void_p(rowidx.data_ptr()), C.c_void_p(val.data_ptr()),
                                   C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), int(accumulate),
                                   _stream(stream)))
    return y


class CuSparse:
    """cuSPARSE CSR FP64 SpMV prepared for repeated calls (alg 0 default,
    1 CSR_ALG1, 2 CSR_ALG2).  Keeps references to the CSR tensors."""

    def __init__(self, m, n, rowptr, colidx, val, alg: int = 0, stream=None):
        self.m, self.n = m, n
        self._keep = (rowptr, colidx, val)
        self._h = C.c_void_p()
        check(load().fl_cusparse_create(C.byref(self._h), m, n, colidx.numel(), C.c_void_p(rowptr.data_ptr()),
                                        C.c_void_p(colidx.data_ptr()), C.c_void_p(val.data_ptr()), int(alg),
                                        _stream(stream)))

    def spmv(self, x, y=None, stream=None):
        torch = _torch()
        _need_cuda(x, torch.float64, self.n, "cusparse spmv x")
        if y is None:
            y = torch.empty(self.m, dtype=torch.float64, device="cuda")
        else:
            _need_cuda(y, torch.float64, self.m, "cusparse spmv y")
        check(load().fl_cusparse_spmv(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                      _stream(stream)))
        return y

    def close(self) -> None:
        if self._h:
            load().fl_cusparse_destroy(self._h)
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
