"""Failure handling on the GPU path: malformed inputs are rejected by
in-bounds validation passes before any kernel could index with them, and an
injected allocation failure surfaces as FL_ERR_ALLOC without poisoning later
calls.  Nothing here faults, traps or hangs the GPU."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_bad_csr_is_rejected(gpu):
    g = load_golden("cfg1")
    m, n, nnz = g["m"], g["n"], g["nnz"]
    ci = g["colidx"].copy()
    ci[17] = n  # column index out of range
    with pytest.raises(gpu.FastLoadError) as e:
        gpu.csr_to_csc(m, n, nnz, g["val"], g["rowptr"], ci)
    assert e.value.code == -1 and "out of range" in str(e.value)
    rp = g["rowptr"].copy()
    rp[5], rp[6] = rp[6], rp[5] - 1  # decreasing row pointer
    with pytest.raises(gpu.FastLoadError):
        gpu.csr_to_csc(m, n, nnz, g["val"], rp, g["colidx"])


def test_bad_colsort_input_is_rejected(gpu):
    g = load_golden("cfg1")
    cnt = g["nnzpercol"].copy()
    cnt[3] += 1  # disagrees with the column pointer
    with pytest.raises(gpu.FastLoadError) as e:
        gpu.ColSort(g["m"], g["n"], g["nnz"], cnt, g["cscptr"], g["cscrow"], g["cscval"], g["x"])
    assert "disagrees" in str(e.value)


def test_bad_format_input_is_rejected(gpu):
    g = load_golden("cfg1")
    snnz = g["sortnnz"][::-1].copy()  # not ascending
    with pytest.raises(gpu.FastLoadError) as e:
        gpu.formatTransform(g["sortrowidx_tmp"], g["sortval_tmp"], snnz, g["nnz"], g["m"], g["n"])
    assert "sorted" in str(e.value)
    snnz = g["sortnnz"].copy()
    snnz[-1] += 1  # sums past nnz
    with pytest.raises(gpu.FastLoadError):
        gpu.formatTransform(g["sortrowidx_tmp"], g["sortval_tmp"], snnz, g["nnz"], g["m"], g["n"])


def test_bad_slide_matrix_is_rejected(gpu):
    g = load_golden("cfg1")
    keys = ["tile_ptr", "tile_len", "tile_colidx", "tile_tall", "tile_format", "countrow", "segmentoffset",
            "sortrowindex", "sortrowidx", "sortval"]
    base = {k: g[k].copy() for k in keys}
    bad = dict(base)
    bad["tile_colidx"] = base["tile_colidx"].copy()
    bad["tile_colidx"][10] += 1  # breaks the staircase
    sm = gpu.SlideMatrix(**bad, tilenum=int(g["tilenum"]), segsum=int(g["segsum"]))
    with pytest.raises(gpu.FastLoadError):
        gpu.FastLoad_spmv(sm, g["nnz"], g["n"], g["m"], g["sortx"], reps=1)
    bad = dict(base)
    bad["sortrowidx"] = base["sortrowidx"].copy()
    bad["sortrowidx"][0] = g["m"]  # row index out of range
    sm = gpu.SlideMatrix(**bad, tilenum=int(g["tilenum"]), segsum=int(g["segsum"]))
    with pytest.raises(gpu.FastLoadError):
        gpu.FastLoad_spmv(sm, g["nnz"], g["n"], g["m"], g["sortx"], reps=1)


def test_injected_allocation_failure_then_recovery(gpu):
    from fastload_gb300 import _lib

    lib = _lib.load()
    g = load_golden("bus_real")
    for k in (1, 3, 7):
        lib.fl_debug_fail_alloc_after(k)
        with pytest.raises(gpu.FastLoadError) as e:
            gpu.csr_to_csc(g["m"], g["n"], g["nnz"], g["val"], g["rowptr"], g["colidx"])
        assert e.value.code == -3
    lib.fl_debug_fail_alloc_after(0)
    t, cv, cr, cp, cnt = gpu.csr_to_csc(g["m"], g["n"], g["nnz"], g["val"], g["rowptr"], g["colidx"])
    np.testing.assert_array_equal(cp, g["cscptr"])
    lib.fl_debug_fail_alloc_after(5)
    with pytest.raises(gpu.FastLoadError):
        gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"], with_reference_arrays=True)
    lib.fl_debug_fail_alloc_after(0)
    p = gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"])
    assert p.info["nnz"] == g["nnz"]
    p.close()


def test_tile_kernel_needs_reference_arrays(gpu):
    import torch

    g = load_golden("cfg1")
    with gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"]) as p:
        xs = torch.zeros(g["n"], dtype=torch.float64, device="cuda")
        with pytest.raises(gpu.FastLoadError):
            p.spmv(xs, kernel=gpu.KERNEL_TILE)
        with pytest.raises(gpu.FastLoadError):
            p.export()


def test_host_call_overlapped_upload_and_its_bounded_wait(gpu):
    """fl_plan_spmv_host uploads the light columns' x on a side stream while
    the heavy band runs; the light items wait for an epoch word that follows
    the copy.  Held back (test hook), the wait runs out after about a second,
    the call reports FL_ERR_NOT_READY, and the next call is correct."""
    import oracle
    from fastload_gb300 import _lib, gen

    lib = _lib.load()
    c = gen.zipf_columns(40000, 1.8, 5000, seed=3)
    ydd = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        assert 0 < p.info["heavy_cols"] < c.n and p.info["items"] > 0
        import torch

        hx = p.permute_x(torch.from_numpy(c.x).cuda()).cpu().numpy()
        for _ in range(3):
            y = p.spmv_host(hx)
            assert oracle.rel_errors(y, ydd)[0] <= 1e-12
        lib.fl_debug_hold_x_upload(1)
        try:
            with pytest.raises(gpu.FastLoadError) as e:
                p.spmv_host(hx)
            assert e.value.code == -6, e.value
        finally:
            lib.fl_debug_hold_x_upload(0)
        y = p.spmv_host(hx)
        assert oracle.rel_errors(y, ydd)[0] <= 1e-12
        p.check()
