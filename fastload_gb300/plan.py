"""Device-resident FastLoad plans (fl_plan_* in include/fastload.h).

A plan builds the FastLoad layout once on the GPU from device CSR/CSC arrays
and keeps it in HBM; SpMV calls then run asynchronously on a CUDA stream.
PyTorch tensors provide the device memory and the current stream.
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np

from ._lib import FastLoadArgumentError, FormInfoC, FormOptsC, PlanInfoC, PlanOptsC, SlideMatrixC, check, load
from .host import SlideMatrix

KERNEL_AUTO = 0
KERNEL_TILE = 1
KERNEL_STREAM = 2
KERNEL_STREAM2 = 3
KERNEL_BUCKET = 4
INPUT_CSR = 0
INPUT_CSC = 1
VALUES_F64 = 0
VALUES_F32 = 1
VALUES_BF16X2 = 2
HEAVY_AUTO, HEAVY_RING, HEAVY_REGS = 0, 1, 2   # FL_HEAVY_*
XSTAGE_AUTO, XSTAGE_GLOBAL = 0, 1            # FL_XSTAGE_*
BAND_AUTO = 0
BAND_NONE = -1
BAND_ALL = -2


PLAN_FILE_MAGIC = b"FLGBPLAN"
_HEADER = struct.Struct("<8sIII9i5Q3QQ")  # 128 bytes, the layout of fl_cache.cu
_HEADER_FIELDS = ("magic", "version", "header_bytes", "byte_order", "m", "n", "nnz", "tilenum", "steps",
                  "with_ref", "heavy", "nforms", "reserved0")
_SECTIONS = ("perm", "sortnnz", "row", "val", "forms")


def plan_file_hash(data: bytes) -> int:
    """Checksum of plan files: 64-bit FNV-1a over little-endian 64-bit words
    (tail zero-padded), xor-ed with the byte count."""
    h = 0xCBF29CE484222325
    pad = (-len(data)) % 8
    for (w,) in struct.iter_unpack("<Q", data + b"\0" * pad):
        h = ((h ^ w) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h ^ len(data)


def plan_file_header(path) -> dict:
    """Header of a plan file (fl_plan_save) as a dict; no GPU needed.  Raises
    ValueError when the file is not a plan file or its header checksum fails."""
    with open(path, "rb") as f:
        raw = f.read(_HEADER.size)
    if len(raw) != _HEADER.size or raw[:8] != PLAN_FILE_MAGIC:
        raise ValueError(f"{path}: not a plan file")
    v = _HEADER.unpack(raw)
    d = dict(zip(_HEADER_FIELDS, v[:13]))
    d["hashes"] = dict(zip(_SECTIONS, v[13:18]))
    if plan_file_hash(raw[:120]) != v[21]:
        raise ValueError(f"{path}: header checksum mismatch")
    return d


def plan_file_sections(path) -> dict:
    """The arrays of a plan file (numpy views of its bytes)."""
    h = plan_file_header(path)
    n, nnz, nf = h["n"], h["nnz"], h["nforms"]
    fi = 3 if h["version"] == 1 else 8  # ints per form: fl_form_opts (version 1: value type, band, y_f32)
    with open(path, "rb") as f:
        f.seek(_HEADER.size)
        out = {"perm": np.fromfile(f, "<i4", n), "sortnnz": np.fromfile(f, "<i4", n),
               "row": np.fromfile(f, "<i4", nnz), "val": np.fromfile(f, "<f8", nnz),
               "forms": np.fromfile(f, "<i4", fi * nf).reshape(nf, fi)}
    return out


def write_plan_file(path, header: dict, sections: dict) -> None:
    """Writes a plan file from a header dict and arrays, recomputing every
    checksum (used to build test inputs)."""
    body = [np.ascontiguousarray(sections[k], dt).tobytes()
            for k, dt in zip(_SECTIONS, ("<i4", "<i4", "<i4", "<f8", "<i4"))]
    hashes = [plan_file_hash(b) for b in body]
    fields = [header[k] for k in _HEADER_FIELDS]
    raw = _HEADER.pack(*fields, *hashes, 0, 0, 0, 0)[:120]
    raw += struct.pack("<Q", plan_file_hash(raw))
    with open(path, "wb") as f:
        f.write(raw)
        for b in body:
            f.write(b)


def _torch():
    import torch

    return torch


def _stream_handle(stream) -> C.c_void_p:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _need_cuda(t, dtype, count: int, what: str) -> None:
    """The kernels index plain device pointers: t must be a contiguous CUDA
    tensor of dtype holding at least count elements."""
    if not (getattr(t, "is_cuda", False) and t.dtype == dtype and t.is_contiguous()):
        raise FastLoadArgumentError(
            f"{what}: needs a contiguous CUDA tensor of {dtype}, got {type(t).__name__} "
            f"{getattr(t, 'dtype', '')} on {getattr(t, 'device', 'host')}")
    if t.numel() < count:
        raise FastLoadArgumentError(f"{what}: needs at least {count} elements, got {t.numel()}")


def _need_host(a, count: int, what: str) -> None:
    """A host array the library copies from or into: C-contiguous float64
    numpy with at least count elements."""
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise FastLoadArgumentError(f"{what}: needs a C-contiguous float64 numpy array, got "
                                    f"{type(a).__name__} {getattr(a, 'dtype', '')}")
    if a.size < count:
        raise FastLoadArgumentError(f"{what}: needs at least {count} elements, got {a.size}")


def _dev(a, dtype):
    """A contiguous CUDA tensor of dtype (uploads numpy input)."""
    torch = _torch()
    if isinstance(a, np.ndarray):
        a = torch.from_numpy(np.ascontiguousarray(a))
    t = a.to(device="cuda", dtype=dtype)
    return t.contiguous()


def convert_values(values, value_type: int = VALUES_F32, stream=None):
    """FP64 values converted on the device to a form's storage type
    (fl_convert_values): a float32 tensor for VALUES_F32, an int32 tensor of
    BF16 hi+lo words (high half bf16(v), low half the 16-bit correction) for
    VALUES_BF16X2."""
    torch = _torch()
    v = _dev(values, torch.float64)
    if value_type not in (VALUES_F32, VALUES_BF16X2):
        raise FastLoadArgumentError(f"convert_values: value type {value_type} (VALUES_F32 or VALUES_BF16X2)")
    out = torch.empty(v.numel(), dtype=torch.float32 if value_type == VALUES_F32 else torch.int32, device=v.device)
    check(load().fl_convert_values(int(value_type), v.numel(), C.c_void_p(v.data_ptr()), C.c_void_p(out.data_ptr()),
                                   _stream_handle(stream)))
    return out


class Plan:
    """FastLoad layout of one matrix resident on the current CUDA device."""

    def __init__(self, handle: C.c_void_p, keep=None):
        self._h = handle
        self._keep = keep
        self._form_kinds = {}  # form id -> (value type, y is FP32)
        self.info = self._info()
        self.m, self.n, self.nnz = self.info["m"], self.info["n"], self.info["nnz"]

    # -- construction ------------------------------------------------------
    @classmethod
    def create(cls, input_format: int, m: int, n: int, ptr, idx, val, with_reference_arrays: bool = False,
               heavy_band: int = 0, stream=None):
        """input_format INPUT_CSR (ptr = row pointer) or INPUT_CSC (ptr =
        column pointer).  heavy_band: -1 no bucketed form, 0 automatic, > 0
        width of the heavy band in columns."""
        torch = _torch()
        if m < 0 or n < 0:
            raise FastLoadArgumentError(f"plan create: negative size (m={m} n={n})")
        p, i, v = _dev(ptr, torch.int32), _dev(idx, torch.int32), _dev(val, torch.float64)
        # the library validates the arrays' contents on the device, reading
        # (m or n) + 1 pointers and nnz values
        npt = (m if input_format == INPUT_CSR else n) + 1
        if p.numel() < npt or v.numel() < i.numel():
            raise FastLoadArgumentError(f"plan create: {p.numel()} pointers (need {npt}), {v.numel()} values for "
                                        f"{i.numel()} indices")
        o = PlanOptsC(int(with_reference_arrays), int(heavy_band))
        h = C.c_void_p()
        check(load().fl_plan_create(C.byref(h), int(input_format), m, n, int(i.numel()), C.c_void_p(p.data_ptr()),
                                    C.c_void_p(i.data_ptr()), C.c_void_p(v.data_ptr()), C.byref(o),
                                    _stream_handle(stream)))
        return cls(h)

    @classmethod
    def from_csr(cls, m: int, n: int, rowptr, colidx, val, with_reference_arrays: bool = False,
                 heavy_band: int = 0, stream=None):
        return cls.create(INPUT_CSR, m, n, rowptr, colidx, val, with_reference_arrays, heavy_band, stream)

    @classmethod
    def from_csc(cls, m: int, n: int, colptr, rowidx, val, with_reference_arrays: bool = False,
                 heavy_band: int = 0, stream=None):
        return cls.create(INPUT_CSC, m, n, colptr, rowidx, val, with_reference_arrays, heavy_band, stream)

    @classmethod
    def from_mtx(cls, path, with_reference_arrays: bool = False, heavy_band: int = 0, stream=None):
        """A plan of a MatrixMarket file, parsed on the GPU (mtx.Mtx) and
        handed over as device CSR without a host round trip."""
        from .mtx import Mtx

        with Mtx.read(path, stream) as mt:
            rp, ci, v = mt.device_pointers()
            o = PlanOptsC(int(with_reference_arrays), int(heavy_band))
            h = C.c_void_p()
            check(load().fl_plan_create(C.byref(h), INPUT_CSR, mt.m, mt.n, mt.nnz, C.c_void_p(rp), C.c_void_p(ci),
                                        C.c_void_p(v), C.byref(o), _stream_handle(stream)))
        return cls(h)

    @classmethod
    def load(cls, path, stream=None):
        """A plan read from a file written by save(): the same layout, heavy
        band and forms, rebuilt on the current device."""
        h = C.c_void_p()
        check(load().fl_plan_load(C.byref(h), str(path).encode(), _stream_handle(stream)))
        return cls(h)

    def save(self, path) -> None:
        """Writes the plan's preprocessed format, options and forms to path."""
        check(load().fl_plan_save(self._h, str(path).encode()))

    # -- queries -------------------------------------------------------------
    def _info(self) -> dict:
        i = PlanInfoC()
        check(load().fl_plan_info_get(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in PlanInfoC._fields_}

    def export(self) -> tuple[SlideMatrix, np.ndarray]:
        """The reference layout (host) and the column permutation."""
        m = SlideMatrixC()
        perm = np.empty(self.n, np.int32)
        lib = load()
        check(lib.fl_plan_export(self._h, C.byref(m), C.c_void_p(perm.ctypes.data)))
        try:
            sm = SlideMatrix._from_c(m, self.nnz)
        finally:
            lib.fl_tile_destroy(C.byref(m))
        return sm, perm

    # -- compute -------------------------------------------------------------
    def permute_x(self, x, out=None, stream=None):
        torch = _torch()
        if out is not None:
            _need_cuda(out, torch.float64, self.n, "permute_x out")
        x = _dev(x, torch.float64)
        _need_cuda(x, torch.float64, self.n, "permute_x x")
        xs = out if out is not None else torch.empty(self.n, dtype=torch.float64, device="cuda")
        check(load().fl_plan_permute_x(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(xs.data_ptr()),
                                       _stream_handle(stream)))
        return xs

    def spmv(self, xs, y=None, accumulate: bool = False, kernel: int = KERNEL_AUTO, stream=None):
        """y = A xs (or y += A xs); xs in sorted column order (permute_x)."""
        torch = _torch()
        _need_cuda(xs, torch.float64, self.n, "spmv xs")
        if y is None:
            y = torch.empty(self.m, dtype=torch.float64, device="cuda")
            accumulate = False
        else:
            _need_cuda(y, torch.float64, self.m, "spmv y")
        check(load().fl_plan_spmv(self._h, C.c_void_p(xs.data_ptr()), C.c_void_p(y.data_ptr()), int(accumulate),
                                  int(kernel), _stream_handle(stream)))
        return y

    def spmv_host(self, xs: np.ndarray, y: np.ndarray | None = None, kernel: int = KERNEL_AUTO, stream=None):
        """Host buffers in and out: H2D of xs, SpMV, D2H of y (synchronous)."""
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        _need_host(xs, self.n, "spmv_host xs")
        if y is None:
            y = np.empty(self.m, np.float64)
        else:
            _need_host(y, self.m, "spmv_host y")
        check(load().fl_plan_spmv_host(self._h, C.c_void_p(xs.ctypes.data), C.c_void_p(y.ctypes.data),
                                       int(kernel), _stream_handle(stream)))
        return y

    def spmv_host_async(self, xs: np.ndarray, y: np.ndarray, kernel: int = KERNEL_AUTO, stream=None) -> np.ndarray:
        """Pipelined host-buffer SpMV: enqueues H2D of xs, y = A xs and D2H
        into y, and returns at once; y is valid after the stream (torch's
        current stream by default) is synchronised.  Consecutive calls
        overlap their copies with the kernels.  xs must hold x when called
        (the upload does not wait for earlier work on the stream); xs and y
        must be C-contiguous float64 arrays that stay alive, unmodified (xs)
        and unread (y) until then; pinned memory (torch pin_memory) lets the
        copies overlap."""
        _need_host(xs, self.n, "spmv_host_async xs")
        _need_host(y, self.m, "spmv_host_async y")
        check(load().fl_plan_spmv_host_async(self._h, C.c_void_p(xs.ctypes.data), C.c_void_p(y.ctypes.data),
                                             int(kernel), _stream_handle(stream)))
        return y

    # -- forms ---------------------------------------------------------------
    def add_form(self, value_type: int = VALUES_F32, heavy_band: int = BAND_AUTO, y_f32: bool = False,
                 light_item: int = 0, heavy_loop: int = HEAVY_AUTO, x_stage: int = XSTAGE_AUTO,
                 unit_warps: int = 0) -> int:
        """Adds a storage form (FP64 / FP32 / BF16 hi+lo values) with the given
        heavy band and build / launch options (fl_form_opts; 0 = automatic);
        returns its id for spmv_form."""
        o = FormOptsC(int(value_type), int(heavy_band), int(y_f32), int(light_item), int(heavy_loop), int(x_stage),
                      int(unit_warps), 0)
        fid = C.c_int(-1)
        check(load().fl_plan_add_form_opts(self._h, C.byref(o), C.byref(fid)))
        self._form_kinds[fid.value] = (int(value_type), bool(y_f32))
        return fid.value

    def form_opts(self, form_id: int) -> dict:
        """The options a form was built with (fl_plan_form_opts_get)."""
        o = FormOptsC()
        check(load().fl_plan_form_opts_get(self._h, int(form_id), C.byref(o)))
        return {k: getattr(o, k) for k, _ in FormOptsC._fields_}

    def set_form_launch(self, form_id: int, heavy_loop: int = HEAVY_AUTO, x_stage: int = XSTAGE_AUTO) -> None:
        """Changes a form's launch options (heavy loop, x staging) in place."""
        check(load().fl_plan_form_set_launch(self._h, int(form_id), int(heavy_loop), int(x_stage)))

    def _kinds(self, form_id: int) -> tuple[int, bool]:
        """(value type, y is FP32) of a form, from the library on first use
        (forms of a loaded plan file)."""
        k = self._form_kinds.get(form_id)
        if k is None:
            i = self.form_info(form_id)
            k = self._form_kinds[form_id] = (int(i["value_type"]), bool(i["y_f32"]))
        return k

    def add_tuned_form(self, value_type: int = VALUES_F32, y_f32: bool = False, model=None) -> tuple[int, str]:
        """Adds the form the learned tuner predicts fastest for this matrix,
        through the C ABI (fl_plan_add_tuned_form: the plan's features through
        the trained network on the GPU; FP32 callers may get BF16 hi+lo
        storage).  Returns (form id, chosen variant's name)."""
        from . import tuner

        path = os.fspath(model or tuner.MODEL)
        fid, var = C.c_int(-1), C.c_int(-1)
        check(load().fl_plan_add_tuned_form(self._h, path.encode(), int(value_type), int(y_f32), C.byref(fid),
                                            C.byref(var)))
        return fid.value, tuner.VARIANTS[var.value]

    def form_info(self, form_id: int) -> dict:
        i = FormInfoC()
        check(load().fl_plan_form_info(self._h, int(form_id), C.byref(i)))
        return {k: getattr(i, k) for k, _ in FormInfoC._fields_}

    def permute_x_k(self, x, k: int = 1, to_f32: bool = False, stream=None):
        """x (n*k, row-interleaved, float64) -> sorted column order, float32
        when to_f32."""
        torch = _torch()
        x = _dev(x, torch.float64).reshape(-1)
        _need_cuda(x, torch.float64, self.n * max(int(k), 0), "permute_x_k x")
        xs = torch.empty(self.n * k, dtype=torch.float32 if to_f32 else torch.float64, device="cuda")
        check(load().fl_plan_permute_x_k(self._h, int(k), int(to_f32), C.c_void_p(x.data_ptr()),
                                         C.c_void_p(xs.data_ptr()), _stream_handle(stream)))
        return xs

    def spmv_form(self, form_id: int, xs, y=None, k: int = 1, accumulate: bool = False, y_f32: bool | None = None,
                  stream=None):
        """y = A xs through a form: xs (n*k, sorted column order, rows of k
        interleaved) is float64 for an FP64 form and float32 otherwise
        (permute_x_k); y (m*k) is float32 when the form accumulates in FP32,
        else float64.  y_f32, when given, must agree with the form."""
        torch = _torch()
        vtype, form_y32 = self._kinds(int(form_id))
        if y_f32 is not None and bool(y_f32) != form_y32:
            raise FastLoadArgumentError(f"spmv_form: form {form_id} has {'an FP32' if form_y32 else 'an FP64'} y")
        kk = max(int(k), 0)
        _need_cuda(xs, torch.float64 if vtype == VALUES_F64 else torch.float32, self.n * kk, "spmv_form xs")
        ydt = torch.float32 if form_y32 else torch.float64
        if y is None:
            y = torch.empty(self.m * k, dtype=ydt, device="cuda")
            accumulate = False
        else:
            _need_cuda(y, ydt, self.m * kk, "spmv_form y")
        check(load().fl_plan_spmv_form(self._h, int(form_id), int(k), C.c_void_p(xs.data_ptr()),
                                       C.c_void_p(y.data_ptr()), int(accumulate), _stream_handle(stream)))
        return y

    def check(self) -> None:
        """Raises FastLoadError if a bounded device wait of the plan's
        kernels expired since the last check (synchronises the device)."""
        check(load().fl_plan_check(self._h))

    def close(self) -> None:
        if self._h:
            load().fl_plan_destroy(self._h)
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
