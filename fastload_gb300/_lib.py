"""ctypes binding of the C ABI in include/fastload.h.

Loading fails loudly (ImportError) when the CUDA library has not been built:
there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_float_p = C.POINTER(C.c_float)


class SlideMatrixC(C.Structure):
    """Same members and order as the reference's slide_matrix
    (src/format.h:6-20) and fl_slide_matrix."""

    _fields_ = [
        ("sortval", c_double_p),
        ("sortrowidx", c_int_p),
        ("tile_ptr", c_int_p),
        ("tile_len", c_int_p),
        ("tile_colidx", c_int_p),
        ("tile_tall", c_int_p),
        ("tile_format", c_int_p),
        ("countrow", c_int_p),
        ("segmentoffset", c_int_p),
        ("sortrowindex", c_int_p),
        ("tilenum", C.c_int),
        ("segsum", C.c_int),
    ]


class PlanInfoC(C.Structure):
    _fields_ = [
        ("m", C.c_int), ("n", C.c_int), ("nnz", C.c_int), ("tilenum", C.c_int), ("steps", C.c_int),
        ("segsum", C.c_int), ("regions", C.c_int), ("items", C.c_int), ("device_bytes", C.c_size_t),
        ("heavy_cols", C.c_int), ("heavy_nnz", C.c_int), ("heavy_slices", C.c_int), ("heavy_padded", C.c_int),
        ("spmv_launches", C.c_int),
    ]


class FormInfoC(C.Structure):
    _fields_ = [("value_type", C.c_int), ("heavy_cols", C.c_int), ("heavy_nnz", C.c_int), ("light_nnz", C.c_int),
                ("y_f32", C.c_int), ("device_bytes", C.c_size_t)]


class FormOptsC(C.Structure):
    """fl_form_opts: build and launch options of a form."""

    _fields_ = [("value_type", C.c_int), ("heavy_band", C.c_int), ("y_f32", C.c_int), ("light_item", C.c_int),
                ("heavy_loop", C.c_int), ("x_stage", C.c_int), ("unit_warps", C.c_int), ("reserved", C.c_int)]


class PlanOptsC(C.Structure):
    _fields_ = [("with_reference_arrays", C.c_int), ("heavy_band", C.c_int), ("reserved", C.c_int * 6)]


class MtxInfoC(C.Structure):
    _fields_ = [("m", C.c_int), ("n", C.c_int), ("nnz", C.c_int), ("nnz_file", C.c_int), ("field", C.c_int),
                ("symmetry", C.c_int), ("is_symmetric", C.c_int), ("exact_path_values", C.c_int),
                ("file_bytes", C.c_size_t)]


# (name, restype, argtypes) of every exported symbol; tests check the .so
# exports each one and that include/fastload.h declares each one.
SIGNATURES = [
    ("fl_last_error", C.c_char_p, []),
    ("fl_version", C.c_char_p, []),
    ("fl_device_count", C.c_int, []),
    ("fl_debug_fail_alloc_after", None, [C.c_int]),
    ("fl_debug_hold_x_upload", None, [C.c_int]),
    ("fl_csr_to_csc", C.c_int, [c_double_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_col_sort", C.c_int, [c_double_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_format_transform", C.c_int, [c_double_p, c_double_p, C.POINTER(SlideMatrixC), C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_int, C.c_int, C.c_int, c_int_p]),
    ("fl_fastload_spmv", C.c_int, [C.POINTER(SlideMatrixC), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_int, c_double_p, c_int_p]),
    ("fl_tile_destroy", None, [C.POINTER(SlideMatrixC)]),
    ("fl_plan_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.POINTER(PlanOptsC), C.c_void_p]),
    ("fl_plan_max_heavy_band", C.c_int, []),
    ("fl_plan_check", C.c_int, [C.c_void_p]),
    ("fl_plan_create_csr", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_void_p]),
    ("fl_plan_create_csc", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_void_p]),
    ("fl_plan_info_get", C.c_int, [C.c_void_p, C.POINTER(PlanInfoC)]),
    ("fl_plan_export", C.c_int, [C.c_void_p, C.POINTER(SlideMatrixC), C.c_void_p]),
    ("fl_plan_permute_x", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_plan_spmv", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("fl_plan_spmv_host", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("fl_plan_spmv_host_async", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("fl_plan_destroy", C.c_int, [C.c_void_p]),
    ("fl_mtx_read", C.c_int, [C.POINTER(C.c_void_p), C.c_char_p, C.c_void_p]),
    ("fl_mtx_info_get", C.c_int, [C.c_void_p, C.POINTER(MtxInfoC)]),
    ("fl_mtx_csr", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    ("fl_mtx_copy_csr", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_mtx_destroy", C.c_int, [C.c_void_p]),
    ("fl_mmio_allinone", C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.POINTER(C.c_int)),
                                   C.POINTER(C.POINTER(C.c_double)), C.c_char_p]),
    ("fl_csc_spmv_naive", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_int, C.c_void_p]),
    ("fl_cusparse_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_void_p]),
    ("fl_cusparse_spmv", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_cusparse_destroy", C.c_int, [C.c_void_p]),
    ("fl_csc_spmv_naive_host", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    ("fl_cusparse_spmv_host", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    ("fl_plan_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("fl_plan_load", C.c_int, [C.POINTER(C.c_void_p), C.c_char_p, C.c_void_p]),
    ("fl_plan_add_form", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("fl_plan_form_info", C.c_int, [C.c_void_p, C.c_int, C.POINTER(FormInfoC)]),
    ("fl_plan_add_form_opts", C.c_int, [C.c_void_p, C.POINTER(FormOptsC), C.POINTER(C.c_int)]),
    ("fl_plan_form_opts_get", C.c_int, [C.c_void_p, C.c_int, C.POINTER(FormOptsC)]),
    ("fl_plan_form_set_launch", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    ("fl_plan_spmv_form", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("fl_plan_permute_x_k", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_convert_values", C.c_int, [C.c_int, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_batch_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p), C.c_int, C.c_int]),
    ("fl_batch_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_long), C.POINTER(C.c_long),
                                C.POINTER(C.c_long), C.POINTER(C.c_int)]),
    ("fl_batch_offsets", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_batch_permute_x", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_batch_spmv", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_batch_spmv_graph", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fl_batch_destroy", C.c_int, [C.c_void_p]),
    ("fl_gen_fill", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                              C.c_ulonglong, C.c_void_p]),
    ("fl_plan_features", C.c_int, [C.c_void_p, C.c_int, c_float_p]),
    ("fl_mlp_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong]),
    ("fl_mlp_num_params", C.c_long, [C.c_void_p]),
    ("fl_mlp_get_params", C.c_int, [C.c_void_p, c_float_p]),
    ("fl_mlp_set_params", C.c_int, [C.c_void_p, c_float_p]),
    ("fl_mlp_forward", C.c_int, [C.c_void_p, c_float_p, C.c_int, c_float_p]),
    ("fl_mlp_grad", C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, C.c_int, c_float_p, c_float_p]),
    ("fl_mlp_train", C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, C.c_int, C.c_int, C.c_float, c_float_p]),
    ("fl_mlp_destroy", C.c_int, [C.c_void_p]),
    ("fl_tuner_variants", C.c_int, [C.POINTER(FormOptsC), C.c_int]),
    ("fl_plan_add_tuned_form", C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]),
    ("fl_col_sort_noalloc", C.c_int, [C.c_int, C.c_int] + [C.c_void_p] * 11),
]

_LIB = None


def load(path: str | None = None) -> C.CDLL:
    """Returns the loaded library, raising ImportError when it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or _build.lib_path()
    if not os.path.exists(p):
        raise ImportError(f"FastLoad GB300 CUDA library not built ({p} missing); "
                          "run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


class FastLoadError(RuntimeError):
    """A library call returned a negative status; .code holds it."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class FastLoadArgumentError(FastLoadError, ValueError):
    """An argument the Python layer rejected before calling the library (a
    tensor or array of the wrong device, type, layout or length, which the
    C ABI's plain pointers could not detect).  Code FL_ERR_ARG."""

    def __init__(self, msg: str):
        super().__init__(-1, msg)


def check(rc: int) -> None:
    if rc != 0:
        msg = load().fl_last_error()
        raise FastLoadError(rc, msg.decode() if msg else "")
