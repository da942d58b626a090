"""CPU oracle for the FastLoad path -- TEST INFRASTRUCTURE ONLY.

Python view of oracle/fl_oracle.c (a plain-C restatement of the reference's
CPU path; see fl_oracle.h for the parity pin).  Only tests/,
__graft_entry__.smoke() and the CPU-baseline leg of bench.py use it, always
as the checker; the fastload_gb300 package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libfastload_ref.so")

_lib = None
_P = C.c_void_p


def _ensure_built() -> None:
    src = [os.path.join(HERE, f) for f in ("fl_oracle.c", "fl_oracle.h", "Makefile")]
    if not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in src):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _ensure_built()
        L = C.CDLL(LIB_PATH)
        I = C.c_int
        sig = {
            "fo_csr2csc": (I, [I, I, I, _P, _P, _P, _P, _P, _P, _P]),
            "fo_col_sort": (I, [I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "fo_count_tiles": (I, [I, _P, C.POINTER(I), C.POINTER(I)]),
            "fo_format_transform": (I, [I, I, _P, _P, _P, I, _P, _P, _P, _P, _P, _P]),
            "fo_tile_classification": (I, [I, I, _P, _P, _P, _P, _P, _P, _P, C.POINTER(I)]),
            "fo_fastload_spmv": (None, [I, _P, _P, _P, _P, _P, _P, _P]),
            "fo_fastload_spmv_omp": (I, [I, _P, _P, _P, _P, _P, _P, _P, I]),
            "fo_csc_spmv": (None, [I, _P, _P, _P, _P, _P]),
            "fo_csr_spmv": (None, [I, _P, _P, _P, _P, _P]),
            "fo_csc_spmv_dd": (None, [I, I, I, _P, _P, _P, _P, _P]),
            "fo_mmio_read": (I, [C.c_char_p, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I), _P, _P, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _i(a):
    return np.ascontiguousarray(a, np.int32)


def _d(a):
    return np.ascontiguousarray(a, np.float64)


def csr2csc(m, n, rowptr, colidx, val):
    """(cscptr, cscrow, cscval, nnzpercol) -- src/coo2csc.h:11-72."""
    rowptr, colidx, val = _i(rowptr), _i(colidx), _d(val)
    nnz = colidx.size
    cp, cr, cv, cnt = np.empty(n + 1, np.int32), np.empty(nnz, np.int32), np.empty(nnz), np.empty(n, np.int32)
    rc = lib().fo_csr2csc(m, n, nnz, _p(rowptr), _p(colidx), _p(val), _p(cp), _p(cr), _p(cv), _p(cnt))
    if rc:
        raise ValueError(f"fo_csr2csc failed ({rc})")
    return cp, cr, cv, cnt


def col_sort(n, nnzpercol, cscptr, cscrow, cscval, x):
    """(perm, sortrowidx_tmp, sortval_tmp, sortnnz, sortx) -- stable order."""
    nnzpercol, cscptr, cscrow, cscval, x = _i(nnzpercol), _i(cscptr), _i(cscrow), _d(cscval), _d(x)
    nnz = cscrow.size
    perm, srow, sval = np.empty(n, np.int32), np.empty(nnz, np.int32), np.empty(nnz)
    snnz, sx = np.empty(n, np.int32), np.empty(n)
    rc = lib().fo_col_sort(n, _p(nnzpercol), _p(cscptr), _p(cscrow), _p(cscval), _p(x), _p(perm), _p(srow),
                           _p(sval), _p(snnz), _p(sx))
    if rc:
        raise ValueError(f"fo_col_sort failed ({rc})")
    return perm, srow, sval, snnz, sx


def format_transform(n, nnz, sortnnz, sortrowidx_tmp, sortval_tmp):
    """Full reference layout as a dict (formattransation + tile_classification)."""
    sortnnz, srow, sval = _i(sortnnz), _i(sortrowidx_tmp), _d(sortval_tmp)
    L = lib()
    h, T = C.c_int(0), C.c_int(0)
    if L.fo_count_tiles(n, _p(sortnnz), C.byref(h), C.byref(T)):
        raise ValueError("fo_count_tiles: tile count overflow")
    T = T.value
    out = {
        "tile_ptr": np.empty(T + 1, np.int32), "tile_len": np.empty(T, np.int32),
        "tile_colidx": np.empty(T, np.int32), "tile_tall": np.empty(T, np.int32),
        "sortrowidx": np.empty(nnz, np.int32), "sortval": np.empty(nnz),
    }
    rc = L.fo_format_transform(n, nnz, _p(sortnnz), _p(srow), _p(sval), T, _p(out["tile_ptr"]),
                               _p(out["tile_len"]), _p(out["tile_colidx"]), _p(out["tile_tall"]),
                               _p(out["sortrowidx"]), _p(out["sortval"]))
    if rc:
        raise ValueError(f"fo_format_transform failed ({rc})")
    fmt, cr = np.empty(T, np.int32), np.empty(T + 1, np.int32)
    seg, sri = np.empty(nnz + 1, np.int32), np.empty(nnz, np.int32)
    S = C.c_int(0)
    L.fo_tile_classification(nnz, T, _p(out["tile_ptr"]), _p(out["tile_len"]), _p(out["sortrowidx"]), _p(fmt),
                             _p(cr), _p(seg), _p(sri), C.byref(S))
    out.update(tile_format=fmt, countrow=cr, segmentoffset=seg[: S.value + 1].copy(), sortrowindex=sri,
               tilenum=T, segsum=S.value, h_count=h.value)
    return out


def build(m, n, rowptr=None, colidx=None, val=None, x=None, csc=None):
    """Whole CPU pipeline from CSR (or a CSC tuple): returns a dict with the
    CSC, the sort results and the layout."""
    if csc is None:
        cp, cr, cv, cnt = csr2csc(m, n, rowptr, colidx, val)
    else:
        cp, cr, cv = (np.asarray(a) for a in csc)
        cnt = np.diff(cp).astype(np.int32)
    xx = np.zeros(n) if x is None else x
    perm, srow, sval, snnz, sx = col_sort(n, cnt, cp, cr, cv, xx)
    lay = format_transform(n, cr.size, snnz, srow, sval)
    lay.update(cscptr=cp, cscrow=cr, cscval=cv, nnzpercol=cnt, perm=perm, sortrowidx_tmp=srow, sortval_tmp=sval,
               sortnnz=snnz, sortx=sx)
    return lay


def fastload_spmv(layout, sortx, m, threads: int = 0):
    """y = A x through the tile loop (FastLoad_CPU.h:19-31); threads > 0 uses
    the OpenMP variant with that many threads (-1: all)."""
    y = np.zeros(m)
    a = [_i(layout["tile_ptr"]), _i(layout["tile_len"]), _i(layout["tile_colidx"]), _i(layout["sortrowidx"]),
         _d(layout["sortval"]), _d(sortx)]
    T = int(layout["tilenum"])
    if threads:
        used = lib().fo_fastload_spmv_omp(T, *[_p(v) for v in a], _p(y), threads if threads > 0 else 0)
        return y, used
    lib().fo_fastload_spmv(T, *[_p(v) for v in a], _p(y))
    return y


def csc_spmv(n, cscptr, cscrow, cscval, x, m):
    y = np.zeros(m)
    lib().fo_csc_spmv(n, _p(_i(cscptr)), _p(_i(cscrow)), _p(_d(cscval)), _p(_d(x)), _p(y))
    return y


def csr_spmv(m, rowptr, colidx, val, x):
    y = np.zeros(m)
    lib().fo_csr_spmv(m, _p(_i(rowptr)), _p(_i(colidx)), _p(_d(val)), _p(_d(x)), _p(y))
    return y


def csc_spmv_dd(m, n, cscptr, cscrow, cscval, x, k: int = 1):
    """Compensated FP64 reference y = A x (x, y row-interleaved for k > 1)."""
    y = np.zeros(m * k)
    lib().fo_csc_spmv_dd(m, n, k, _p(_i(cscptr)), _p(_i(cscrow)), _p(_d(cscval)), _p(_d(x)), _p(y))
    return y if k == 1 else y.reshape(m, k)


def mmio_read(path):
    """(m, n, nnz, is_symmetric, rowptr, colidx, val) of a coordinate .mtx
    file, read as the reference's mmio_allinone reads it."""
    m, n, nnz, sym = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    L = lib()
    rc = L.fo_mmio_read(str(path).encode(), C.byref(m), C.byref(n), C.byref(nnz), C.byref(sym), None, None, None)
    if rc:
        raise ValueError(f"fo_mmio_read failed ({rc}) for {path}")
    rp, ci, v = np.empty(m.value + 1, np.int32), np.empty(max(nnz.value, 1), np.int32), np.empty(max(nnz.value, 1))
    rc = L.fo_mmio_read(str(path).encode(), C.byref(m), C.byref(n), C.byref(nnz), C.byref(sym), _p(rp), _p(ci), _p(v))
    if rc:
        raise ValueError(f"fo_mmio_read failed ({rc}) for {path}")
    return m.value, n.value, nnz.value, sym.value, rp, ci[:nnz.value], v[:nnz.value]


def rel_errors(y, yref):
    """(normwise ||y - y*||_2 / ||y*||_2, max|y - y*| / ||y*||_inf)."""
    y, yref = np.asarray(y, np.float64), np.asarray(yref, np.float64)
    d = y - yref
    n2 = float(np.linalg.norm(yref))
    ninf = float(np.max(np.abs(yref))) if yref.size else 0.0
    return (float(np.linalg.norm(d)) / n2 if n2 else float(np.linalg.norm(d)),
            float(np.max(np.abs(d))) / ninf if ninf else float(np.max(np.abs(d)) if d.size else 0.0))


def bf16x2_split(v):
    """Numpy restatement of the BF16 hi+lo value storage (no reference
    counterpart: the storage form is this engine's).  Returns the 32-bit
    words: high half hi = bf16(v) rounded to nearest even from the FP64
    value, low half the signed 16-bit correction d = round((v - hi) / hi *
    2^22) clamped to +-32767 (d = 0 when hi is zero, non-finite or below
    2^-100 in magnitude)."""
    v = np.asarray(v, np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        m, e = np.frexp(v)  # v = m 2^e, 0.5 <= |m| < 1
        # 8 significant bits, round half to even (np.rint); below the normal
        # range the BF16 spacing is 2^-133
        hf = np.where(e >= -125, np.ldexp(np.rint(np.ldexp(m, 8)), e - 8), np.rint(np.ldexp(v, 133)) * 2.0 ** -133)
        hf = np.where(np.isfinite(v), hf, v)
        hi_b = hf.astype(np.float32).view(np.uint32)  # exact; overflow to +-inf past the BF16 range
        hf = hi_b.view(np.float32).astype(np.float64)
        ok = (np.abs(hf) >= 2.0 ** -100) & np.isfinite(hf)
        d = np.where(ok, np.rint((v - hf) / np.where(ok, hf, 1.0) * 2.0 ** 22), 0.0)
    d = np.clip(d, -32767, 32767).astype(np.int16)
    return hi_b | d.view(np.uint16).astype(np.uint32)


def bf16x2_value(words):
    """Decoded FP32 value of BF16 hi+lo words, as the kernels decode it:
    fma(hi * 2^-22, d, hi), rounded once to FP32."""
    w = np.asarray(words, np.uint32)
    hi = (w & np.uint32(0xFFFF0000)).view(np.float32).astype(np.float64)
    d = (w & np.uint32(0xFFFF)).astype(np.uint16).view(np.int16).astype(np.float64)
    return (hi * 2.0 ** -22 * d + hi).astype(np.float32)
