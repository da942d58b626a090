"""CUDA path against the golden fixtures and the CPU oracle, through the C ABI.

Layout (CSC, column sort, every slide_matrix array) must be bit-exact.  y
must match the exactly rounded A x to a normwise relative error of 1e-12
(the FP64 bound of the workload; atomics reorder the additions) and exactly
when values and x are small integers, as in the reference's own check."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT, golden_names, load_golden

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
LAYOUT_KEYS = ["tile_ptr", "tile_len", "tile_colidx", "tile_tall", "tile_format", "countrow", "segmentoffset",
               "sortrowindex", "sortrowidx", "sortval"]
INTEGER_CASES = {"bus_i10", "spmv9", "runs", "dups"}
KERNELS = ["KERNEL_AUTO", "KERNEL_STREAM", "KERNEL_STREAM2", "KERNEL_TILE"]


def assert_y(y, g, name):
    if name in INTEGER_CASES:
        np.testing.assert_array_equal(y, g["y_exact"])
    else:
        nw, mx = oracle.rel_errors(y, g["y_exact"])
        assert nw <= FP64_TOL and mx <= FP64_TOL, (name, nw, mx)


@pytest.mark.parametrize("name", golden_names())
def test_reference_calls_match_golden(gpu, name):
    g = load_golden(name)
    m, n, nnz = g["m"], g["n"], g["nnz"]
    t, cv, cr, cp, cnt = gpu.csr_to_csc(m, n, nnz, g["val"], g["rowptr"], g["colidx"])
    np.testing.assert_array_equal(cp, g["cscptr"])
    np.testing.assert_array_equal(cr, g["cscrow"])
    np.testing.assert_array_equal(cv, g["cscval"])
    np.testing.assert_array_equal(cnt, g["nnzpercol"])
    t, srow, sval, snnz, sx = gpu.ColSort(m, n, nnz, cnt, cp, cr, cv, g["x"])
    np.testing.assert_array_equal(snnz, g["sortnnz"])
    np.testing.assert_array_equal(sx, g["sortx"])
    np.testing.assert_array_equal(srow, g["sortrowidx_tmp"])
    np.testing.assert_array_equal(sval, g["sortval_tmp"])
    ta, tb, sm, h = gpu.formatTransform(srow, sval, snnz, nnz, m, n)
    assert sm.tilenum == g["tilenum"] and sm.segsum == g["segsum"]
    for k in LAYOUT_KEYS:
        np.testing.assert_array_equal(getattr(sm, k), g[k], err_msg=k)
    y, ms, bad = gpu.FastLoad_spmv(sm, nnz, n, m, sx, y_golden=g["y_exact"], reps=3)
    assert_y(y, g, name)
    if name in INTEGER_CASES:
        assert bad == 0


@pytest.mark.parametrize("name", golden_names())
def test_plan_matches_golden(gpu, name):
    import torch

    g = load_golden(name)
    m, n = g["m"], g["n"]
    with gpu.Plan.from_csr(m, n, g["rowptr"], g["colidx"], g["val"], with_reference_arrays=True) as p:
        assert p.info["tilenum"] == g["tilenum"]
        sm, perm = p.export()
        np.testing.assert_array_equal(perm, g["perm"])
        for k in LAYOUT_KEYS:
            np.testing.assert_array_equal(getattr(sm, k), g[k], err_msg=k)
        xs = p.permute_x(torch.from_numpy(g["x"]).cuda())
        np.testing.assert_array_equal(xs.cpu().numpy(), g["sortx"])
        for kern in KERNELS:
            y = p.spmv(xs, kernel=getattr(gpu, kern))
            torch.cuda.synchronize()
            assert_y(y.cpu().numpy(), g, f"{name}/{kern}")
        y2 = p.spmv_host(g["sortx"])
        assert_y(y2, g, name)
        # accumulate: y += A x on top of y = A x gives 2 A x
        y = p.spmv(xs)
        p.spmv(xs, y=y, accumulate=True)
        assert_y(y.cpu().numpy() / 2, g, name)


@pytest.mark.parametrize("name", ["cfg1", "bus_real", "zipf_small"])
def test_plan_from_csc_matches_csr(gpu, name):
    g = load_golden(name)
    a = gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"], with_reference_arrays=True)
    b = gpu.Plan.from_csc(g["m"], g["n"], g["cscptr"], g["cscrow"], g["cscval"], with_reference_arrays=True)
    sa, pa = a.export()
    sb, pb = b.export()
    np.testing.assert_array_equal(pa, pb)
    for k in LAYOUT_KEYS:
        np.testing.assert_array_equal(getattr(sa, k), getattr(sb, k))
    a.close()
    b.close()


def test_fastload_spmv_accepts_the_reference_cpu_layout(gpu):
    """A slide_matrix produced by the reference's own code (the golden) runs
    through FastLoad_spmv unchanged."""
    g = load_golden("cfg1")
    sm = gpu.SlideMatrix(**{k: g[k] for k in LAYOUT_KEYS}, tilenum=int(g["tilenum"]), segsum=int(g["segsum"]))
    y, ms, bad = gpu.FastLoad_spmv(sm, g["nnz"], g["n"], g["m"], g["sortx"], reps=2)
    assert_y(y, g, "cfg1")


def _full_size_case(kind):
    from fastload_gb300 import gen

    if kind == "zipf":
        return gen.zipf_columns(1 << 20, 1.8, 50000, seed=2)
    return gen.laplacian7(128, seed=4)


@pytest.mark.parametrize("kind", ["zipf", "laplacian"])
def test_full_size_layout_and_result(gpu, kind):
    """Full benchmark sizes: the GPU layout equals the oracle's bit for bit;
    y is within 1e-12 of the compensated oracle; linearity and the column-sum
    checksum hold."""
    import torch

    c = _full_size_case(kind)
    ref = oracle.build(c.m, c.n, csc=(c.colptr, c.rowidx, c.val), x=c.x)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val, with_reference_arrays=True) as p:
        sm, perm = p.export()
        np.testing.assert_array_equal(perm, ref["perm"])
        assert sm.tilenum == ref["tilenum"] and sm.segsum == ref["segsum"]
        for k in LAYOUT_KEYS:
            np.testing.assert_array_equal(getattr(sm, k), ref[k], err_msg=k)
        x = torch.from_numpy(c.x).cuda()
        xs = p.permute_x(x)
        ydd = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
        for kern in KERNELS:
            y = p.spmv(xs, kernel=getattr(gpu, kern)).cpu().numpy()
            nw, mx = oracle.rel_errors(y, ydd)
            assert nw <= FP64_TOL and mx <= FP64_TOL, (kern, nw, mx)
        # linearity: A(x1 + x2) = A x1 + A x2
        x2 = torch.linspace(-1, 1, c.n, dtype=torch.float64, device="cuda")
        xs2 = p.permute_x(x2)
        ya = p.spmv(xs + xs2).cpu().numpy()
        yb = (p.spmv(xs) + p.spmv(xs2)).cpu().numpy()
        assert np.linalg.norm(ya - yb) <= 1e-12 * np.linalg.norm(ya)
        # checksum: sum_i (A x)_i = sum_c x_c colsum_c
        colsum = np.add.reduceat(c.val, c.colptr[:-1]) if c.nnz else np.zeros(c.n)
        colsum[np.diff(c.colptr) == 0] = 0.0
        y = p.spmv(xs).cpu().numpy()
        assert abs(y.sum() - np.dot(colsum, c.x)) <= 1e-9 * np.abs(c.val).sum()


def test_plan_build_is_deterministic(gpu):
    g = load_golden("zipf_small")
    outs = []
    for _ in range(2):
        with gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"], with_reference_arrays=True) as p:
            outs.append(p.export())
    for k in LAYOUT_KEYS:
        np.testing.assert_array_equal(getattr(outs[0][0], k), getattr(outs[1][0], k))


def test_dropin_driver_runs_the_main_cu_sequence(gpu, tmp_path):
    """tests/dropin/main_dropin.cpp (main.cu's call sequence on
    fastload_compat.h) prints the reference's PASS line on 1138_bus."""
    from fastload_gb300 import _build

    exe = str(tmp_path / "dropin")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "dropin", "main_dropin.cpp"), "-o", exe,
                    "-L", _build.LIBDIR, "-lfastload_gb300", f"-Wl,-rpath,{_build.LIBDIR}"], check=True)
    g = load_golden("bus_i10")
    path = tmp_path / "bus.bin"
    with open(path, "wb") as f:
        np.array([g["m"], g["n"], g["nnz"]], np.int32).tofile(f)
        g["rowptr"].astype(np.int32).tofile(f)
        g["colidx"].astype(np.int32).tofile(f)
    r = subprocess.run([exe, str(path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Check FASTLOAD GPU PASS!" in r.stdout
    assert "Check FASTLOAD CPU PASS!" in r.stdout
    assert f"tilenum {g['tilenum']}" in r.stdout
    assert "BASIC CSC GPU PASS!" in r.stdout
    assert "cuSPARSE test PASSED!" in r.stdout
    # main.cu:40's read of a .mtx file, parsed on the GPU
    mtx = os.path.join(ROOT, "tests", "golden", "mtx", "real_symmetric.mtx")
    r = subprocess.run([exe, mtx], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "nnz =13" in r.stdout
    assert "Check FASTLOAD GPU PASS!" in r.stdout and "Check FASTLOAD CPU PASS!" in r.stdout


@pytest.mark.parametrize("name", golden_names())
def test_bucketed_form_matches_golden(gpu, name):
    """The bucketed kernel (light columns streamed, heavy band in row slices
    with x staged in shared memory) with a forced band of up to 64 columns."""
    import torch

    g = load_golden(name)
    m, n = g["m"], g["n"]
    band = min(n, 64) & ~1
    with gpu.Plan.from_csr(m, n, g["rowptr"], g["colidx"], g["val"], heavy_band=band if band else -1) as p:
        if band and g["nnz"]:
            assert p.info["heavy_cols"] == band
        xs = p.permute_x(torch.from_numpy(g["x"]).cuda())
        for kern in (gpu.KERNEL_AUTO,) + ((gpu.KERNEL_BUCKET,) if p.info["heavy_cols"] else ()):
            y = p.spmv(xs, kernel=kern)
            assert_y(y.cpu().numpy(), g, f"{name}/bucket")
        p.check()


def test_bucketed_form_unaligned_x_uses_plain_staging(gpu):
    """x whose band slice is not 16-byte aligned cannot be staged by the bulk
    copy; the kernel then copies it with ordinary loads.  Same result."""
    import torch

    g = load_golden("zipf_small")
    with gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"], heavy_band=512) as p:
        buf = torch.zeros(g["n"] + 1, dtype=torch.float64, device="cuda")
        xs_al = p.permute_x(torch.from_numpy(g["x"]).cuda())
        buf[1:] = xs_al
        xs_un = buf[1:]  # 8-byte offset
        ya = p.spmv(xs_al, kernel=gpu.KERNEL_BUCKET).cpu().numpy()
        yb = p.spmv(xs_un, kernel=gpu.KERNEL_BUCKET).cpu().numpy()
        assert_y(ya, g, "aligned")
        assert_y(yb, g, "unaligned")
        p.check()


@pytest.mark.parametrize("kind", ["zipf", "laplacian"])
def test_full_size_bucketed(gpu, kind):
    import torch

    c = _full_size_case(kind)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        if kind == "zipf":
            assert p.info["heavy_cols"] == 16384
            assert p.info["heavy_nnz"] > 0.8 * c.nnz
        else:
            # no dense columns, but a stencil's x gathers have locality: every
            # column goes into the band as row slices
            assert p.info["heavy_cols"] == c.n
        xs = p.permute_x(torch.from_numpy(c.x).cuda())
        ydd = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
        y = p.spmv(xs).cpu().numpy()
        nw, mx = oracle.rel_errors(y, ydd)
        assert nw <= FP64_TOL and mx <= FP64_TOL, (nw, mx)
        p.check()


def test_automatic_layout_rule(gpu):
    """The default plan: a band of dense columns when there are any; with
    none, row slices over every column when x gathers have locality or rows
    are skewed, and the plain FastLoad stream for uniformly random rows.
    Every choice computes the same product."""
    import torch

    from fastload_gb300 import gen, sweep

    cases = [("random rows", gen.diag_poisson(20000, seed=3), 0),
             ("random rows, 1M+ nonzeros, 5 a column", gen.diag_poisson(1 << 18, seed=3), "all"),
             ("stencil", gen.laplacian7(24), "all"),
             ("skewed rows", sweep._gen_family(4, 20000, 3.0), "all"),
             ("dense columns", gen.zipf_columns(40000, 1.8, 5000, seed=3), "band")]
    for name, c, expect in cases:
        with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
            h = p.info["heavy_cols"]
            if expect == "all":
                assert h == c.n, (name, h)
            elif expect == "band":
                assert 0 < h < c.n, (name, h)
            else:
                assert h == 0, (name, h)
            xs = p.permute_x(torch.from_numpy(c.x).cuda())
            ydd = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
            for kern in (gpu.KERNEL_AUTO, gpu.KERNEL_STREAM):
                y = p.spmv(xs, kernel=kern).cpu().numpy()
                assert oracle.rel_errors(y, ydd)[0] <= FP64_TOL, (name, kern)
            p.check()


def test_back_to_back_spmv_overwrites_y(gpu):
    """y = A x launched back to back with no synchronisation in between (the
    y-zeroing and SpMV launches overlap their start-up): every call
    overwrites whatever y held, accumulate adds, and the reported launch
    count matches the layout (one launch when the band owns every row)."""
    import torch

    from fastload_gb300 import gen, sweep

    cases = [("random rows", gen.diag_poisson(20000, seed=3), 2),
             ("stencil", gen.laplacian7(24), 1),
             ("skewed rows", sweep._gen_family(4, 20000, 3.0), None),
             ("dense columns", gen.zipf_columns(40000, 1.8, 5000, seed=3), 2)]
    for name, c, launches in cases:
        ydd = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
        with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
            if launches is not None:
                assert p.info["spmv_launches"] == launches, (name, p.info)
            xs = p.permute_x(torch.from_numpy(c.x).cuda())
            y = torch.full((c.m,), float("nan"), dtype=torch.float64, device="cuda")
            y2 = torch.full((c.m,), float("nan"), dtype=torch.float64, device="cuda")
            for _ in range(3):
                p.spmv(xs, y)
                p.spmv(xs, y, accumulate=True)
                p.spmv(xs, y2)
            fid = p.add_form(gpu.VALUES_F64)
            y3 = torch.full((c.m,), float("nan"), dtype=torch.float64, device="cuda")
            for _ in range(3):
                p.spmv_form(fid, xs, y3)
            torch.cuda.synchronize()
            assert oracle.rel_errors(y.cpu().numpy() / 2, ydd)[0] <= FP64_TOL, name
            assert oracle.rel_errors(y2.cpu().numpy(), ydd)[0] <= FP64_TOL, name
            assert oracle.rel_errors(y3.cpu().numpy(), ydd)[0] <= FP64_TOL, name
            p.check()


def test_dropin_fastload_spmv_runs_the_bucketed_kernel(gpu):
    """The reference's call sequence (csr_to_csc -> ColSort ->
    formatTransform -> FastLoad_spmv) on a matrix with dense columns: the
    drop-in FastLoad_spmv builds the bucketed split from the slide_matrix and
    its product matches the oracle; on integer data it is exact (the
    reference's own check counts no mismatch)."""
    import scipy.sparse as sp

    from fastload_gb300 import gen

    c = gen.zipf_columns(40000, 1.8, 5000, seed=3)
    A = sp.csc_matrix((c.val, c.rowidx, c.colptr), shape=(c.m, c.n)).tocsr()
    rp, ci = A.indptr.astype(np.int32), A.indices.astype(np.int32)
    for integer in (False, True):
        val = np.round(A.data * 4) if integer else A.data
        x = np.round(c.x * 8) if integer else c.x
        t, cv, cr, cp, cnt = gpu.csr_to_csc(c.m, c.n, len(val), val, rp, ci)
        t, srow, sval, snnz, sx = gpu.ColSort(c.m, c.n, len(val), cnt, cp, cr, cv, x)
        ta, tb, sm, h = gpu.formatTransform(srow, sval, snnz, len(val), c.m, c.n)
        ydd = oracle.csc_spmv_dd(c.m, c.n, cp, cr, cv, x)
        y, ms, bad = gpu.FastLoad_spmv(sm, len(val), c.n, c.m, sx, y_golden=ydd, reps=3)
        assert ms > 0
        if integer:
            np.testing.assert_array_equal(y, ydd)
            assert bad == 0
        else:
            assert oracle.rel_errors(y, ydd)[0] <= FP64_TOL
