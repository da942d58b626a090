"""fl_col_sort_noalloc: the column sort for callers that may not allocate
device memory (for instance a plugin living inside an application that has
already claimed the whole GPU for its own memory pool, or a latency-critical
caller that cannot pay for the synchronisation cudaMalloc/cudaFree cause).

It runs on device arrays the caller owns and keeps its scratch in one static
device array of the library, so its results must equal those of the regular
host-buffer entry point fl_col_sort exactly (the column sort only moves
integers and copies values).  Two calls in a row, the second on a smaller
matrix, check that the contents the shared scratch keeps from one call never
leak into the next.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc_sort(lib, g):
    import torch

    n, nnz = int(g["n"]), int(g["nnz"])
    dev = dict(cnt=torch.from_numpy(g["nnzpercol"].astype(np.int32)).cuda(),
               ptr=torch.from_numpy(g["cscptr"].astype(np.int32)).cuda(),
               row=torch.from_numpy(g["cscrow"].astype(np.int32)).cuda(),
               val=torch.from_numpy(g["cscval"].astype(np.float64)).cuda(),
               x=torch.from_numpy(g["x"].astype(np.float64)).cuda())
    out = dict(perm=torch.full((n,), -7, dtype=torch.int32, device="cuda"),
               snnz=torch.full((n,), -7, dtype=torch.int32, device="cuda"),
               srow=torch.full((max(nnz, 1),), -7, dtype=torch.int32, device="cuda"),
               sval=torch.full((max(nnz, 1),), np.nan, dtype=torch.float64, device="cuda"),
               sx=torch.full((n,), np.nan, dtype=torch.float64, device="cuda"))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.fl_col_sort_noalloc(n, nnz, _ptr(dev["cnt"]), _ptr(dev["ptr"]), _ptr(dev["row"]), _ptr(dev["val"]),
                                 _ptr(dev["x"]), _ptr(out["perm"]), _ptr(out["snnz"]), _ptr(out["srow"]),
                                 _ptr(out["sval"]), _ptr(out["sx"]), stream)
    assert rc == 0, lib.fl_last_error()
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def test_noalloc_col_sort_matches_col_sort_twice(gpu):
    from fastload_gb300 import _lib

    lib = _lib.load()
    for name in ("cfg1", "zipf_small", "bus_real"):  # largest first, then smaller ones
        g = load_golden(name)
        nnz = int(g["nnz"])
        t, srow, sval, snnz, sx = gpu.ColSort(g["m"], g["n"], nnz, g["nnzpercol"], g["cscptr"], g["cscrow"],
                                              g["cscval"], g["x"])
        got = _noalloc_sort(lib, g)
        np.testing.assert_array_equal(got["snnz"], snnz)
        np.testing.assert_array_equal(got["srow"][:nnz], srow)
        np.testing.assert_array_equal(got["sval"][:nnz], sval)
        np.testing.assert_array_equal(got["sx"], sx)
        np.testing.assert_array_equal(got["perm"], g["perm"])


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    from fastload_gb300 import _lib

    lib = _lib.load()
    n = 262144 + 1
    rc = lib.fl_col_sort_noalloc(n, 0, *([None] * 10), None)
    assert rc == -1
    msg = lib.fl_last_error().decode()
    assert "FL_NOALLOC_MAX_COLS" in msg and str(n) in msg


def _case(c):
    deg = np.diff(c.colptr).astype(np.int32)
    return {"m": c.m, "n": c.n, "nnz": c.nnz, "nnzpercol": deg, "cscptr": c.colptr, "cscrow": c.rowidx,
            "cscval": c.val, "x": c.x, "perm": np.argsort(deg, kind="stable").astype(np.int32)}


def test_noalloc_multi_tile_sizes_twice(gpu):
    """At the size limit (262,144 columns: 64 radix tiles of 4,096 columns,
    so the digit histograms and the column-pointer scan span several blocks
    and the scan recurses), then on about 20,000 columns (5 tiles) with the
    same shared scratch: both equal fl_col_sort bit for bit, and the
    permutation is the stable order of the column counts."""
    from fastload_gb300 import _lib, gen

    lib = _lib.load()
    cases = (gen.zipf_columns(262144, 1.8, 5000, seed=31), gen.zipf_columns(20011, 1.5, 3000, seed=32))
    assert cases[0].n == 262144  # FL_NOALLOC_MAX_COLS
    for c in cases:
        g = _case(c)
        t, srow, sval, snnz, sx = gpu.ColSort(g["m"], g["n"], g["nnz"], g["nnzpercol"], g["cscptr"], g["cscrow"],
                                              g["cscval"], g["x"])
        got = _noalloc_sort(lib, g)
        np.testing.assert_array_equal(got["perm"], g["perm"])
        np.testing.assert_array_equal(got["snnz"], snnz)
        np.testing.assert_array_equal(got["srow"][:g["nnz"]], srow)
        np.testing.assert_array_equal(got["sval"][:g["nnz"]], sval)
        np.testing.assert_array_equal(got["sx"], sx)
