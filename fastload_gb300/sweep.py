"""Sweep driver: FastLoad against its comparators over synthetic matrix
families, one CSV row per matrix.

Covers what the reference's profiling/test.sh (run ./test over sizes x
sparsities), profiling/ncu-tests.sh (the same grid under ncu) and
profiling/data.py (collect the printed times into profiling_data.csv) do
together:

* family "random": the test.cu grid -- M = N in {1000, ..., 12000}, an entry
  kept when a uniform draw in [0, 100) exceeds the sparsity (test.cu:30-43),
  values U[0, 1); seeded numpy instead of rand();
* the synthetic families of the benchmarks (Poisson columns, Zipf degrees,
  7-point Laplacian, banded, block diagonal, skewed rows).

Columns keep data.py's names and units (ms, GFLOP/s) for the fields it
defines, then add the device-plan kernel time, algorithmic GB/s, % of the
measured HBM peak, cuSPARSE CSR and the normwise difference against the naive
kernel.  Every time is a CUDA-event time except the reference-compatible
host calls, which report their own (ColSort, formatTransform,
FastLoad_spmv, as the reference prints them).

    python -m fastload_gb300.sweep --out sweep.csv                 # full grid
    python -m fastload_gb300.sweep --families random --sizes 1000,4000 --sparsities 50,90
    python -m fastload_gb300.sweep --list                          # case names
    python -m fastload_gb300.sweep --case random_s50_n4000         # one case (e.g. under ncu)
"""
from __future__ import annotations

import argparse
import csv
import json
import os
import sys
import time

import numpy as np

SIZES = (1000, 2000, 4000, 6000, 8000, 10000, 12000)
SPARSITIES = (10, 20, 30, 40, 50, 60, 70, 80, 90, 95)
REF_HEADERS = [
    "sparsity", "matrix_size", "M", "N", "nnz", "CSC_SpMV_Time", "Memory_H2D_Time", "Kernel_Time",
    "Memory_D2H_Time", "GFLOPS", "FastLoad_sort_time", "FastLoad_format_transform_time",
    "FastLoad_format_classification_time", "FastLoad_total_preprocessing_time", "FastLoad_GPU_PASS_time",
    "FastLoad_GFLOPS", "FastLoad_memcpy_H2D_time", "FastLoad_memcpy_D2H_time",
]
EXTRA_HEADERS = ["family", "case", "plan_kernel", "plan_kernel_ms", "plan_gbs", "plan_pct_of_peak",
                 "plan_gflops", "cusparse_ms", "cusparse_gflops", "rel_diff_vs_naive"]


def random_csc(size: int, sparsity: int, seed: int):
    """test.cu:30-43 with numpy: keep (i, j) when U{0..99} > sparsity."""
    from .gen import CSC

    rng = np.random.default_rng(seed)
    keep = rng.integers(0, 100, (size, size), dtype=np.int16) > sparsity  # [column, row]
    col, row = np.nonzero(keep)
    colptr = np.zeros(size + 1, np.int64)
    np.cumsum(np.bincount(col, minlength=size), out=colptr[1:])
    val = rng.random(row.size)
    x = rng.uniform(-1, 1, size)
    return CSC(size, size, colptr.astype(np.int32), row.astype(np.int32), val, x)


def cases(families, sizes, sparsities):
    """(family, case name, sparsity or "", size, builder) for the grid."""
    from . import gen

    out = []
    if "random" in families:
        for sp in sparsities:
            for n in sizes:
                out.append(("random", f"random_s{sp}_n{n}", sp, n,
                            (lambda sp=sp, n=n: random_csc(n, sp, seed=1000 * sp + n))))
    if "poisson" in families:
        for n in (1 << 12, 1 << 16, 1 << 20):
            out.append(("poisson", f"poisson_n{n}", "", n, lambda n=n: gen.diag_poisson(n, seed=1)))
    if "zipf" in families:
        for n in (1 << 16, 1 << 18, 1 << 20):
            out.append(("zipf", f"zipf_n{n}", "", n, lambda n=n: gen.zipf_columns(n, 1.8, 50000, seed=2)))
    if "laplacian" in families:
        for N in (32, 64, 128):
            out.append(("laplacian", f"laplacian_{N}cubed", "", N ** 3, lambda N=N: gen.laplacian7(N)))
    for fam, fid, param in (("banded", 2, 64.0), ("block", 3, 256.0), ("rowskew", 4, 3.0)):
        if fam in families:
            for n in (1 << 16, 1 << 20):
                out.append((fam, f"{fam}_n{n}", "", n, lambda n=n, fid=fid, param=param:
                            _gen_family(fid, n, param)))
    return out


def _gen_family(family: int, n: int, param: float):
    """Columns of Poisson(8)+1 degrees filled by the device generator
    (fl_gen_fill) for families 2 banded, 3 block diagonal, 4 skewed rows."""
    import ctypes as C

    import torch

    from . import _lib
    from .gen import CSC

    rng = np.random.default_rng(family * 7 + n)
    d = rng.poisson(8, n) + 1
    if family in (2, 3):
        d = np.minimum(d, int(param))
    colptr = np.concatenate([[0], np.cumsum(d)]).astype(np.int32)
    nnz = int(colptr[-1])
    cp = torch.from_numpy(colptr).cuda()
    rows = torch.empty(nnz, dtype=torch.int32, device="cuda")
    vals = torch.empty(nnz, dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().fl_gen_fill(family, n, n, C.c_void_p(cp.data_ptr()), C.c_void_p(rows.data_ptr()),
                                       C.c_void_p(vals.data_ptr()), param, C.c_ulonglong(family + n), None))
    return CSC(n, n, colptr, rows.cpu().numpy(), vals.cpu().numpy(), rng.uniform(-1, 1, n))


def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _mean_ms(fn, reps, before=None):
    import torch

    a, b = _events()
    for _ in range(2):
        if before:
            before()
        fn()
    ts = []
    for _ in range(reps):
        if before:
            before()
        a.record()
        fn()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    return float(np.mean(ts))


def measure(family, name, sparsity, size, build, reps=20, peak=None) -> dict:
    import torch

    import fastload_gb300 as fl
    from fastload_gb300 import compare

    c = build()
    m, n, nnz = c.m, c.n, c.nnz
    row = {"family": family, "case": name, "sparsity": sparsity, "matrix_size": size, "M": m, "N": n, "nnz": nnz}
    flops = 2.0 * nnz
    # naive CSC with its copies (test.cu: H2D, kernel, D2H)
    a, b = _events()
    a.record()
    cp = torch.from_numpy(c.colptr).cuda()
    cr = torch.from_numpy(c.rowidx).cuda()
    cv = torch.from_numpy(c.val).cuda()
    x = torch.from_numpy(c.x).cuda()
    b.record()
    b.synchronize()
    row["Memory_H2D_Time"] = a.elapsed_time(b)
    y = torch.zeros(m, dtype=torch.float64, device="cuda")
    k_ms = _mean_ms(lambda: compare.csc_spmv_naive(m, cp, cr, cv, x, y=y, accumulate=True), reps, before=y.zero_)
    row["Kernel_Time"] = k_ms
    hy = torch.empty(m, dtype=torch.float64).pin_memory()
    a.record()
    hy.copy_(y, non_blocking=True)
    b.record()
    b.synchronize()
    row["Memory_D2H_Time"] = a.elapsed_time(b)
    row["CSC_SpMV_Time"] = row["Memory_H2D_Time"] + k_ms + row["Memory_D2H_Time"]
    row["GFLOPS"] = flops / (k_ms * 1e-3) / 1e9
    y_naive = y.double().cpu().numpy()

    # FastLoad through the reference-compatible host calls (their own times)
    t_sort, srow, sval, snnz, sx = fl.ColSort(m, n, nnz, np.diff(c.colptr), c.colptr, c.rowidx, c.val, c.x)
    t_tran, t_class, sm, _ = fl.formatTransform(srow, sval, snnz, nnz, m, n)
    row["FastLoad_sort_time"] = t_sort
    row["FastLoad_format_transform_time"] = t_tran
    row["FastLoad_format_classification_time"] = t_class
    row["FastLoad_total_preprocessing_time"] = t_sort + t_tran + t_class
    _, pass_ms, _ = fl.FastLoad_spmv(sm, nnz, n, m, sx, None, reps=reps)
    row["FastLoad_GPU_PASS_time"] = pass_ms
    row["FastLoad_GFLOPS"] = flops / (pass_ms * 1e-3) / 1e9

    # the device plan (automatic kernel), its copies and the difference
    with fl.Plan.from_csc(m, n, c.colptr, c.rowidx, c.val) as p:
        xs = p.permute_x(x)
        kern = "bucket" if p.info["heavy_cols"] else "stream"
        pm = _mean_ms(lambda: p.spmv(xs, y, accumulate=True), reps, before=y.zero_)
        hx = torch.from_numpy(np.ascontiguousarray(xs.cpu().numpy())).pin_memory()
        a.record()
        xs.copy_(hx, non_blocking=True)
        b.record()
        b.synchronize()
        row["FastLoad_memcpy_H2D_time"] = a.elapsed_time(b)
        p.spmv(xs, y)
        a.record()
        hy.copy_(y, non_blocking=True)
        b.record()
        b.synchronize()
        row["FastLoad_memcpy_D2H_time"] = a.elapsed_time(b)
        d = np.linalg.norm(hy.numpy() - y_naive) / max(np.linalg.norm(y_naive), 1e-300)
        p.check()
    B = nnz * 12 + (n + 1) * 4 + n * 8 + m * 8
    row.update(plan_kernel=kern, plan_kernel_ms=pm, plan_gbs=B / (pm * 1e-3) / 1e9,
               plan_pct_of_peak=(100.0 * B / (pm * 1e-3) / 1e9 / peak) if peak else "",
               plan_gflops=flops / (pm * 1e-3) / 1e9, rel_diff_vs_naive=d)
    # cuSPARSE CSR (the reference's second comparator)
    try:
        import scipy.sparse as sp

        A = sp.csc_matrix((c.val, c.rowidx, c.colptr), shape=(m, n)).tocsr()
        rp = torch.from_numpy(A.indptr.astype(np.int32)).cuda()
        ci = torch.from_numpy(A.indices.astype(np.int32)).cuda()
        v = torch.from_numpy(A.data).cuda()
        with compare.CuSparse(m, n, rp, ci, v) as cs:
            cm = _mean_ms(lambda: cs.spmv(x, y=y), reps)
        row.update(cusparse_ms=cm, cusparse_gflops=flops / (cm * 1e-3) / 1e9)
    except fl.FastLoadError as e:
        row.update(cusparse_ms="", cusparse_gflops="")
        print(f"[sweep] cuSPARSE unavailable: {e}", file=sys.stderr)
    return row


def _peak():
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--families", default="random,poisson,zipf,laplacian,banded,block,rowskew")
    ap.add_argument("--sizes", default=",".join(map(str, SIZES)), help="sizes of the random family")
    ap.add_argument("--sparsities", default=",".join(map(str, SPARSITIES)), help="sparsities (%%) of the random family")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--out", default="sweep.csv")
    ap.add_argument("--case", default=None, help="run only this case")
    ap.add_argument("--list", action="store_true", help="print the case names and exit")
    a = ap.parse_args(argv)
    fams = set(a.families.split(","))
    grid = cases(fams, [int(s) for s in a.sizes.split(",")], [int(s) for s in a.sparsities.split(",")])
    if a.list:
        for g in grid:
            print(g[1])
        return 0
    if a.case:
        grid = [g for g in grid if g[1] == a.case]
        if not grid:
            print(f"no case {a.case}", file=sys.stderr)
            return 2
    peak = _peak()
    headers = REF_HEADERS + EXTRA_HEADERS
    t0 = time.time()
    with open(a.out, "w", newline="") as f:
        w = csv.DictWriter(f, fieldnames=headers)
        w.writeheader()
        for fam, name, sp, size, build in grid:
            r = measure(fam, name, sp, size, build, a.reps, peak)
            w.writerow({k: (f"{v:.6g}" if isinstance(v, float) else v) for k, v in r.items()})
            f.flush()
            print(f"[sweep] {name}: nnz={r['nnz']} naive {r['Kernel_Time']:.4f} ms, FastLoad plan "
                  f"{r['plan_kernel_ms']:.4f} ms ({r['plan_gbs']:.0f} GB/s), cuSPARSE {r.get('cusparse_ms', '')} ms"
                  f" [{time.time() - t0:.0f} s]", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
