"""Batches: many FastLoad matrices through one persistent launch
(fl_batch_* in include/fastload.h), optionally replayed as a CUDA graph."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, load
from .plan import VALUES_F32, Plan, _dev, _need_cuda, _stream_handle, _torch


class Batch:
    """Stacked FastLoad layouts of several plans (y and x stacked in order)."""

    def __init__(self, plans: list[Plan], value_type: int = VALUES_F32, y_f32: bool = True):
        arr = (C.c_void_p * max(len(plans), 1))(*[p._h for p in plans])
        h = C.c_void_p()
        check(load().fl_batch_create(C.byref(h), len(plans), arr, int(value_type), int(y_f32)))
        self._h = h
        self.value_type, self.y_f32 = int(value_type), bool(y_f32)
        cnt, nitems = C.c_int(), C.c_int()
        m, n, z = C.c_long(), C.c_long(), C.c_long()
        check(load().fl_batch_info(self._h, C.byref(cnt), C.byref(m), C.byref(n), C.byref(z), C.byref(nitems)))
        self.count, self.m, self.n, self.nnz, self.items = cnt.value, m.value, n.value, z.value, nitems.value
        self.m_off = np.empty(self.count + 1, np.int32)
        self.n_off = np.empty(self.count + 1, np.int32)
        check(load().fl_batch_offsets(self._h, C.c_void_p(self.m_off.ctypes.data), C.c_void_p(self.n_off.ctypes.data)))

    def permute_x(self, x, stream=None):
        torch = _torch()
        x = _dev(x, torch.float64)
        _need_cuda(x, torch.float64, self.n, "batch permute_x x")
        xs = torch.empty(self.n, dtype=torch.float64 if self.value_type == 0 else torch.float32, device="cuda")
        check(load().fl_batch_permute_x(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(xs.data_ptr()),
                                        _stream_handle(stream)))
        return xs

    def _y(self, xs, y):
        """Checks xs (float64 for FP64 values, else float32; n stacked
        columns) and y (float32 when y_f32, else float64; m stacked rows),
        allocating y when it is None."""
        torch = _torch()
        _need_cuda(xs, torch.float64 if self.value_type == 0 else torch.float32, self.n, "batch xs")
        ydt = torch.float32 if self.y_f32 else torch.float64
        if y is None:
            y = torch.empty(self.m, dtype=ydt, device="cuda")
        else:
            _need_cuda(y, ydt, self.m, "batch y")
        return y

    def spmv(self, xs, y=None, stream=None):
        y = self._y(xs, y)
        check(load().fl_batch_spmv(self._h, C.c_void_p(xs.data_ptr()), C.c_void_p(y.data_ptr()),
                                   _stream_handle(stream)))
        return y

    def spmv_graph(self, xs, y=None, stream=None):
        y = self._y(xs, y)
        check(load().fl_batch_spmv_graph(self._h, C.c_void_p(xs.data_ptr()), C.c_void_p(y.data_ptr()),
                                         _stream_handle(stream)))
        return y

    def close(self):
        if self._h:
            load().fl_batch_destroy(self._h)
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
