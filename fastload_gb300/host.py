"""Reference-named host API over the C ABI.

Mirrors the reference's host calls for the FastLoad path -- csr_to_csc
(src/csr2csc_cuda.h:51), ColSort (src/ColSort_GPU.h:46), formatTransform
(src/formatTransform_GPU.h:289) and FastLoad_spmv (src/FastLoad_GPU.h:275) --
with the same argument order and meaning.  Output arrays are returned as numpy
arrays instead of being written through out-parameters; where the reference
prints an error and continues, these raise FastLoadError.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import FastLoadArgumentError, FastLoadError, SlideMatrixC, check, load

__all__ = ["SlideMatrix", "csr_to_csc", "ColSort", "formatTransform", "FastLoad_spmv", "FastLoadError"]


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


@dataclass
class SlideMatrix:
    """The reference's slide_matrix (src/format.h:6-20) as numpy arrays."""

    sortval: np.ndarray
    sortrowidx: np.ndarray
    tile_ptr: np.ndarray
    tile_len: np.ndarray
    tile_colidx: np.ndarray
    tile_tall: np.ndarray
    tile_format: np.ndarray
    countrow: np.ndarray
    segmentoffset: np.ndarray
    sortrowindex: np.ndarray
    tilenum: int
    segsum: int

    @classmethod
    def _from_c(cls, m: SlideMatrixC, nnz: int) -> "SlideMatrix":
        T, S = m.tilenum, m.segsum

        def grab(ptr, count, dt):
            if count == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dt, copy=True)

        return cls(
            sortval=grab(m.sortval, nnz, np.float64), sortrowidx=grab(m.sortrowidx, nnz, np.int32),
            tile_ptr=grab(m.tile_ptr, T + 1, np.int32), tile_len=grab(m.tile_len, T, np.int32),
            tile_colidx=grab(m.tile_colidx, T, np.int32), tile_tall=grab(m.tile_tall, T, np.int32),
            tile_format=grab(m.tile_format, T, np.int32), countrow=grab(m.countrow, T + 1, np.int32),
            segmentoffset=grab(m.segmentoffset, S + 1, np.int32), sortrowindex=grab(m.sortrowindex, nnz, np.int32),
            tilenum=T, segsum=S)

    def to_c(self) -> tuple[SlideMatrixC, list]:
        """A C struct pointing into these arrays (keep the returned list alive)."""
        keep = [_f64(self.sortval), _i32(self.sortrowidx), _i32(self.tile_ptr), _i32(self.tile_len),
                _i32(self.tile_colidx), _i32(self.tile_tall), _i32(self.tile_format), _i32(self.countrow),
                _i32(self.segmentoffset), _i32(self.sortrowindex)]
        d = C.POINTER(C.c_double)
        i = C.POINTER(C.c_int)
        m = SlideMatrixC(keep[0].ctypes.data_as(d), *[k.ctypes.data_as(i) for k in keep[1:]],
                         int(self.tilenum), int(self.segsum))
        return m, keep

    def fields(self) -> dict:
        return {k: getattr(self, k) for k in ("sortval", "sortrowidx", "tile_ptr", "tile_len", "tile_colidx",
                                              "tile_tall", "tile_format", "countrow", "segmentoffset",
                                              "sortrowindex", "tilenum", "segsum")}


def csr_to_csc(m: int, n: int, nnz: int, csr_val, csr_row_ptr, csr_col_ind):
    """CSR (m x n) -> CSC on the GPU.  Returns (time_ms, csc_val, csc_row_ind,
    csc_col_ptr, nnzpercol); rows ascending within each column."""
    lib = load()
    v, rp, ci = _f64(csr_val), _i32(csr_row_ptr), _i32(csr_col_ind)
    if rp.size != m + 1 or v.size < nnz or ci.size < nnz:
        raise FastLoadError(-1, "csr_to_csc: array sizes do not match m/nnz")
    cv = np.empty(nnz, np.float64)
    cr = np.empty(nnz, np.int32)
    cp = np.empty(n + 1, np.int32)
    npc = np.empty(n, np.int32)
    t = C.c_double(0)
    check(lib.fl_csr_to_csc(C.byref(t), m, n, nnz, _p(v), _p(rp), _p(ci), _p(cv), _p(cr), _p(cp), _p(npc)))
    return t.value, cv, cr, cp, npc


def ColSort(rowA: int, colA: int, nnz: int, nnzPerCol, cscColPtr, cscRowIdx, cscVal, x):
    """Stable column sort by nonzeros per column on the GPU.  Returns
    (time_ms, sortrowidx_tmp, sortval_tmp, sortnnz_tmp, sortx)."""
    lib = load()
    cnt, cp, cr, cv = _i32(nnzPerCol), _i32(cscColPtr), _i32(cscRowIdx), _f64(cscVal)
    xx = None if x is None else _f64(x)
    if cnt.size < colA or cp.size < colA + 1 or cr.size < nnz or cv.size < nnz or (xx is not None and xx.size < colA):
        raise FastLoadError(-1, "ColSort: array sizes do not match colA/nnz")
    srow = np.empty(nnz, np.int32)
    sval = np.empty(nnz, np.float64)
    snnz = np.empty(colA, np.int32)
    sx = None if xx is None else np.empty(colA, np.float64)
    t = C.c_double(0)
    check(lib.fl_col_sort(C.byref(t), rowA, colA, nnz, _p(cnt), _p(cp), _p(cr), _p(cv), _p(srow), _p(sval),
                          _p(snnz), _p(xx), _p(sx)))
    return t.value, srow, sval, snnz, sx


def formatTransform(sortrowidx_tmp, sortval_tmp, sortnnz_tmp, nnz: int, rowA: int, colA: int):
    """FastLoad tile layout on the GPU.  Returns (time_tran_ms,
    time_class_ms, SlideMatrix, h_count)."""
    lib = load()
    srow, sval, snnz = _i32(sortrowidx_tmp), _f64(sortval_tmp), _i32(sortnnz_tmp)
    if srow.size < nnz or sval.size < nnz or snnz.size < colA:
        raise FastLoadError(-1, "formatTransform: array sizes do not match nnz/colA")
    m = SlideMatrixC()
    ta, tb = C.c_double(0), C.c_double(0)
    h = C.c_int(0)
    check(lib.fl_format_transform(C.byref(ta), C.byref(tb), C.byref(m), _p(srow), _p(sval), _p(snnz), nnz, rowA,
                                  colA, C.byref(h)))
    try:
        sm = SlideMatrix._from_c(m, nnz)
    finally:
        lib.fl_tile_destroy(C.byref(m))
    return ta.value, tb.value, sm, h.value


def FastLoad_spmv(matrix: SlideMatrix, nnz: int, colA: int, rowA: int, x_sorted, y_golden=None, reps: int = 100):
    """y = A x on the GPU from a host slide_matrix.  Returns (y, ms_per_spmv,
    mismatches) where mismatches counts |y_golden - y| > 0.01|y| (0 when no
    golden is given)."""
    xs = _f64(x_sorted)
    if xs.size < colA:
        raise FastLoadError(-1, "FastLoad_spmv: x_sorted shorter than colA")
    yg = None if y_golden is None else _f64(y_golden)
    if yg is not None and yg.size < rowA:
        raise FastLoadArgumentError(f"FastLoad_spmv: y_golden has {yg.size} entries, rowA={rowA}")
    # the library copies these many entries of each array to the device
    T = int(matrix.tilenum)
    need = {"sortval": nnz, "sortrowidx": nnz, "tile_ptr": T + 1, "tile_len": T, "tile_colidx": T}
    short = [f"{k} ({np.size(getattr(matrix, k))} < {v})" for k, v in need.items() if np.size(getattr(matrix, k)) < v]
    if short:
        raise FastLoadArgumentError("FastLoad_spmv: slide_matrix arrays shorter than tilenum/nnz: " + ", ".join(short))
    lib = load()
    y = np.empty(rowA, np.float64)
    cm, keep = matrix.to_c()
    ms = C.c_double(0)
    bad = C.c_int(0)
    check(lib.fl_fastload_spmv(C.byref(cm), nnz, colA, rowA, _p(xs), _p(y), _p(yg), reps, C.byref(ms),
                               C.byref(bad)))
    del keep
    return y, ms.value, bad.value
