"""The reference's own CPU path, compiled from its sources into oracle/_ref/
(TEST INFRASTRUCTURE ONLY; see ref_shim.cpp).  Available only on a machine
that holds the reference sources; callers skip when it is absent."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import REF_LIB_PATH

_P = C.c_void_p
_lib = None


def available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(REF_LIB_PATH)
        I, IP = C.c_int, C.POINTER(C.c_int)
        sig = {
            "ref_mmio_read": (I, [C.c_char_p, IP, IP, IP, IP, _P, _P, _P]),
            "ref_csr2csc": (None, [I, I, I, _P, _P, _P, _P, _P, _P, _P]),
            "ref_col_sort": (None, [I, I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "ref_layout_build": (C.c_void_p, [I, I, I, _P, _P, _P]),
            "ref_layout_sizes": (None, [C.c_void_p, IP, IP]),
            "ref_layout_get": (None, [C.c_void_p, I] + [_P] * 10),
            "ref_fastload_cpu": (None, [C.c_void_p, I, I, I, _P, _P, _P]),
            "ref_layout_free": (None, [C.c_void_p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def mmio_read(path: str):
    """(m, n, nnz, is_symmetric, rowptr, colidx, val) via mmio_allinone."""
    m, n, nnz, sym = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    rc = lib().ref_mmio_read(path.encode(), C.byref(m), C.byref(n), C.byref(nnz), C.byref(sym), None, None, None)
    if rc:
        raise OSError(f"mmio_allinone failed ({rc}) for {path}")
    rp, ci, v = np.empty(m.value + 1, np.int32), np.empty(nnz.value, np.int32), np.empty(nnz.value)
    lib().ref_mmio_read(path.encode(), C.byref(m), C.byref(n), C.byref(nnz), C.byref(sym), _p(rp), _p(ci), _p(v))
    return m.value, n.value, nnz.value, sym.value, rp, ci, v


def csr2csc(m, n, rowptr, colidx, val):
    rowptr, colidx, val = (np.ascontiguousarray(a) for a in (rowptr.astype(np.int32), colidx.astype(np.int32),
                                                              val.astype(np.float64)))
    nnz = colidx.size
    cp, cr, cv, cnt = np.empty(n + 1, np.int32), np.empty(nnz, np.int32), np.empty(nnz), np.empty(n, np.int32)
    lib().ref_csr2csc(m, n, nnz, _p(rowptr), _p(colidx), _p(val), _p(cp), _p(cr), _p(cv), _p(cnt))
    return cp, cr, cv, cnt


def col_sort(n, nnzpercol, cscptr, cscrow, cscval, x):
    """The reference's std::sort column sort: (sortrowidx_tmp, sortval_tmp,
    sortnnz, sortx); tie order unspecified."""
    a = [np.ascontiguousarray(v) for v in (nnzpercol.astype(np.int32), cscptr.astype(np.int32),
                                           cscrow.astype(np.int32), cscval.astype(np.float64),
                                           x.astype(np.float64))]
    nnz = a[2].size
    srow, sval, snnz, sx = np.empty(nnz, np.int32), np.empty(nnz), np.empty(n, np.int32), np.empty(n)
    lib().ref_col_sort(n, nnz, *[_p(v) for v in a[:4]], _p(a[4]), _p(srow), _p(sval), _p(snnz), _p(sx))
    return srow, sval, snnz, sx


def layout(m, n, nnz, sortrowidx_tmp, sortval_tmp, sortnnz, sortx=None, y_golden=None):
    """formattransation + tile_classification (+ FastLoad_cpu when sortx is
    given): dict of the slide_matrix arrays, tilenum, segsum and y."""
    srow = np.ascontiguousarray(sortrowidx_tmp, np.int32)
    sval = np.ascontiguousarray(sortval_tmp, np.float64)
    snnz = np.ascontiguousarray(sortnnz, np.int32)
    L = lib()
    h = L.ref_layout_build(m, n, nnz, _p(srow), _p(sval), _p(snnz))
    try:
        T, S = C.c_int(), C.c_int()
        L.ref_layout_sizes(h, C.byref(T), C.byref(S))
        T, S = T.value, S.value
        out = {
            "tile_ptr": np.empty(T + 1, np.int32), "tile_len": np.empty(T, np.int32),
            "tile_colidx": np.empty(T, np.int32), "tile_tall": np.empty(T, np.int32),
            "tile_format": np.empty(T, np.int32), "countrow": np.empty(T + 1, np.int32),
            "segmentoffset": np.empty(S + 1, np.int32), "sortrowindex": np.empty(nnz, np.int32),
            "sortrowidx": np.empty(nnz, np.int32), "sortval": np.empty(nnz),
        }
        L.ref_layout_get(h, nnz, *[_p(out[k]) for k in ("tile_ptr", "tile_len", "tile_colidx", "tile_tall",
                                                          "tile_format", "countrow", "segmentoffset",
                                                          "sortrowindex", "sortrowidx", "sortval")])
        out["tilenum"], out["segsum"] = T, S
        if sortx is not None:
            y = np.zeros(m)
            yg = np.zeros(m) if y_golden is None else np.ascontiguousarray(y_golden, np.float64)
            L.ref_fastload_cpu(h, nnz, m, n, _p(np.ascontiguousarray(sortx, np.float64)), _p(y), _p(yg))
            out["y"] = y
        return out
    finally:
        L.ref_layout_free(h)
