"""Generates the golden fixtures in tests/golden/*.npz.

Every expected array comes from the reference's own CPU code (compiled from
its sources into oracle/_ref/ by `make -C oracle ref`) or from plain numpy /
exact rational arithmetic -- never from this repository's oracle or CUDA
library, which the fixtures then check:

* csr2csc                 -> reference csr2csc (src/coo2csc.h:11-72)
* column permutation       -> numpy stable argsort of the column counts (the
                              order of thrust::sort_by_key in ColSort_GPU.h:101)
* layout (all slide_matrix arrays, tilenum, segsum)
                           -> reference formattransation + tile_classification
                              (src/coo2csc.h:132-448) on the stable-sorted arrays
* y                        -> reference FastLoad_cpu (src/FastLoad_CPU.h:2-46)
* y_exact                  -> exactly rounded A x (Python fractions)
* ref_pipeline_*           -> the reference's own pipeline with its CPU
                              col_sort (std::sort), for the record

Inputs: the reference's bundled Data/1138_bus.mtx (read with the reference's
mmio_allinone), the 9x9 matrix of spmv.cu (parsed from that file), seeded
synthetic matrices and small edge cases.  Run from the repo root:

    make -C oracle all ref REF_SRC=<checkout>/src &&
        FL_REFERENCE=<checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import re
import sys
from fractions import Fraction

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fastload_gb300 import gen  # noqa: E402  (generators only, no CUDA)
from oracle import ref  # noqa: E402

REF = os.environ.get("FL_REFERENCE")  # the reference checkout (its Data/ and spmv.cu); required
OUT = os.path.dirname(os.path.abspath(__file__))


def exact_y(m, n, colptr, rowidx, val, x):
    acc = [Fraction(0)] * m
    for c in range(n):
        xc = Fraction(float(x[c]))
        for p in range(colptr[c], colptr[c + 1]):
            acc[rowidx[p]] += Fraction(float(val[p])) * xc
    return np.array([float(a) for a in acc])


def case(name, m, n, rowptr, colidx, val, x, note, exact=True):
    rowptr, colidx = np.asarray(rowptr, np.int32), np.asarray(colidx, np.int32)
    val, x = np.asarray(val, np.float64), np.asarray(x, np.float64)
    nnz = colidx.size
    cp, cr, cv, cnt = ref.csr2csc(m, n, rowptr, colidx, val)
    perm = np.argsort(cnt, kind="stable").astype(np.int32)
    snnz = cnt[perm]
    sx = x[perm]
    srow = np.concatenate([cr[cp[c]:cp[c + 1]] for c in perm]) if nnz else np.zeros(0, np.int32)
    sval = np.concatenate([cv[cp[c]:cp[c + 1]] for c in perm]) if nnz else np.zeros(0)
    lay = ref.layout(m, n, nnz, srow, sval, snnz, sortx=sx, y_golden=None)
    # the reference's own end-to-end CPU pipeline (unstable std::sort)
    rrow, rval, rnnz, rsx = ref.col_sort(n, cnt, cp, cr, cv, x)
    rlay = ref.layout(m, n, nnz, rrow, rval, rnnz)
    d = dict(m=m, n=n, nnz=nnz, rowptr=rowptr, colidx=colidx, val=val, x=x,
             cscptr=cp, cscrow=cr, cscval=cv, nnzpercol=cnt,
             perm=perm, sortnnz=snnz, sortx=sx, sortrowidx_tmp=srow.astype(np.int32), sortval_tmp=sval,
             y=lay.pop("y"), ref_pipeline_tilenum=rlay["tilenum"], ref_pipeline_segsum=rlay["segsum"],
             ref_sortnnz=rnnz, note=note)
    for k, v in lay.items():
        d[k] = v
    if exact:
        d["y_exact"] = exact_y(m, n, cp, cr, cv, x)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **d)
    print(f"{name:12s} m={m} n={n} nnz={nnz} tilenum={lay['tilenum']} segsum={lay['segsum']} "
          f"fmt={np.bincount(lay['tile_format'], minlength=3).tolist()}")


def from_csc(c: gen.CSC):
    rp, ci, v = c.to_csr()
    return c.m, c.n, rp, ci, v, c.x


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("make_golden.py: set FL_REFERENCE to the reference checkout (its Data/ and spmv.cu are read)")
    rng = np.random.default_rng(20261203)
    # 1. the reference's bundled matrix, run the way main.cu runs it
    m, n, nnz, sym, rp, ci, v = ref.mmio_read(os.path.join(REF, "Data", "1138_bus.mtx"))
    case("bus_i10", m, n, rp, ci, (np.arange(nnz) % 10).astype(float), (np.arange(n) % 10).astype(float),
         "Data/1138_bus.mtx; val=i%10 (main.cu:68-69), x=i%10 (main.cu:93-96)")
    case("bus_real", m, n, rp, ci, v, rng.uniform(-1, 1, n), "Data/1138_bus.mtx with its own values, x U[-1,1]")
    # 2. the 9x9 known-answer matrix of spmv.cu (its golden there is A^T 1; ours is exact A x)
    txt = open(os.path.join(REF, "spmv.cu")).read()
    block = re.search(r"temp_A\[9\]\[9\]\s*=\s*\{(.*?)\};", txt, re.S).group(1)
    A = np.array([[float(t) for t in re.findall(r"-?\d+", row)] for row in re.findall(r"\{([^{}]*)\}", block)])
    assert A.shape == (9, 9)
    r, c = np.nonzero(A)
    rp9 = np.concatenate([[0], np.cumsum(np.bincount(r, minlength=9))])
    case("spmv9", 9, 9, rp9, c, A[r, c], np.ones(9), "9x9 matrix of spmv.cu:140-150, x = 1")
    # 3. the small FP64 benchmark configuration: n=4096, diag + Poisson(4)
    m, n, rp, ci, v, x = from_csc(gen.diag_poisson(4096, 4.0, seed=1))
    case("cfg1", m, n, rp, ci, v, x, "n=4096 diag + Poisson(4) distinct rows, U[-1,1] values and x, seed 1")
    # 4. miniature Zipf and Laplacian matrices
    m, n, rp, ci, v, x = from_csc(gen.zipf_columns(3000, 1.8, 500, seed=5))
    case("zipf_small", m, n, rp, ci, v, x, "n=3000 Zipf(1.8) degrees capped at 500, seed 5")
    m, n, rp, ci, v, x = from_csc(gen.laplacian7(8, seed=6))
    case("lap8", m, n, rp, ci, v, x, "7-point Laplacian on an 8^3 grid, seed 6")
    # 5. edge cases
    case("n1", 1, 1, [0, 1], [0], [2.5], [-3.0], "1x1")
    case("empty", 5, 7, np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0), np.ones(7), "nnz = 0")

    def random_csr(m, n, maxdeg, p_empty, seed):
        g = np.random.default_rng(seed)
        rows, cols = [], []
        for col in range(n):
            if g.random() < p_empty:
                continue
            k = int(g.integers(1, maxdeg + 1))
            rr = np.sort(g.choice(m, size=min(k, m), replace=False))
            rows += rr.tolist()
            cols += [col] * len(rr)
        rows, cols = np.array(rows, np.int64), np.array(cols, np.int64)
        order = np.lexsort((cols, rows))
        rows, cols = rows[order], cols[order]
        rp = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=m))])
        return rp, cols, g.uniform(-1, 1, rows.size), g.uniform(-1, 1, n)

    for w in (31, 32, 33, 63, 64, 65):
        rp, ci, v, x = random_csr(50, w, 6, 0.1, seed=w)
        case(f"w{w}", 50, w, rp, ci, v, x, f"n={w} columns (tile width boundary), degrees 1..6, 10% empty")
    rp, ci, v, x = random_csr(40, 70, 5, 0.5, seed=7)
    case("empty_cols", 40, 70, rp, ci, v, x, "half the columns empty")
    rp, ci, v, x = random_csr(300, 77, 9, 0.0, seed=8)
    case("rect_tall", 300, 77, rp, ci, v, x, "m=300 > n=77")
    rp, ci, v, x = random_csr(50, 200, 4, 0.0, seed=9)
    case("rect_wide", 50, 200, rp, ci, v, x, "m=50 < n=200")
    # one dense column among sparse ones
    g = np.random.default_rng(10)
    ent = [(r, 7, g.uniform(-1, 1)) for r in range(100)]
    for col in range(50):
        if col != 7:
            for r in g.choice(100, size=int(g.integers(0, 4)), replace=False):
                ent.append((int(r), col, g.uniform(-1, 1)))
    cc = gen.from_csr_lists(100, 50, ent, x=g.uniform(-1, 1, 50))
    m, n, rp, ci, v, x = from_csc(cc)
    case("dense_col", m, n, rp, ci, v, x, "column 7 dense (100 nonzeros)")
    # one dense row: every column holds row 5 -> full tiles of one run (format 1)
    ent = [(5, col, g.uniform(-1, 1)) for col in range(96)]
    for col in range(0, 96, 3):
        ent.append((int(g.integers(6, 64)), col, g.uniform(-1, 1)))
    cc = gen.from_csr_lists(64, 96, ent, x=g.uniform(-1, 1, 96))
    m, n, rp, ci, v, x = from_csc(cc)
    case("dense_row", m, n, rp, ci, v, x, "row 5 dense: format-1 tiles")
    # long runs inside tiles: level l of every column is row l, with breaks
    ent = []
    for col in range(256):
        k = 1 + col % 5
        for l in range(k):
            ent.append((l if col % 7 else l + 1, col, float(1 + (col + l) % 9)))
    cc = gen.from_csr_lists(8, 256, ent, x=(np.arange(256) % 7).astype(float))
    m, n, rp, ci, v, x = from_csc(cc)
    case("runs", m, n, rp, ci, v, x, "runs of equal rows across tiles (formats 1 and 2)")
    # duplicate entries in the CSR
    rp = np.array([0, 3, 5, 6])
    ci = np.array([1, 1, 2, 0, 0, 2])
    case("dups", 3, 3, rp, ci, np.array([1.0, 2.0, 3.0, 4.0, 5.0, 6.0]), np.array([1.0, 10.0, 100.0]),
         "duplicate (row, col) entries kept in CSR order")


if __name__ == "__main__":
    if not ref.available():
        sys.exit("oracle/_ref/libfastload_ref.so missing: run `make -C oracle ref` on a machine with the reference")
    main()
