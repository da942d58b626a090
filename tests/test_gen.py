"""The seeded generators that stand in for the reference's SuiteSparse
inputs: CSC invariants (rows ascending and distinct inside every column, as
src/csr2csc_cuda.h produces them), value ranges, and the sizes that the
benchmark and the parity cases are quoted on."""
import numpy as np

import bench
from fastload_gb300 import gen


def check_csc(c, dtype=np.float64):
    assert c.colptr.dtype == np.int32 and c.rowidx.dtype == np.int32
    assert c.colptr.size == c.n + 1 and c.colptr[0] == 0 and c.colptr[-1] == c.nnz
    assert np.all(np.diff(c.colptr) >= 0)
    if c.nnz:
        assert c.rowidx.min() >= 0 and c.rowidx.max() < c.m
        col = np.repeat(np.arange(c.n, dtype=np.int64), np.diff(c.colptr))
        keys = col * c.m + c.rowidx
        assert np.all(np.diff(keys) > 0), "rows must ascend strictly inside each column"
    assert c.val.dtype == dtype and c.x.dtype == dtype and c.x.size == c.n
    assert np.all(np.isfinite(c.val)) and np.all(np.abs(c.x) <= 1.0)


def test_bench_matrix_is_the_quoted_workload():
    c = bench.make_workload()
    check_csc(c)
    assert c.m == c.n == 1 << 20
    assert c.nnz == 26_978_074  # Zipf(1.8) degrees capped at 50,000, seed 2
    assert c.degrees().max() == 50_000
    assert bench.algorithmic_bytes(c.m, c.n, c.nnz) == 344_708_412  # B per SpMV in the bench line


def test_laplacian7_is_symmetric_with_the_stencil_count():
    N = 128
    c = gen.laplacian7(N)
    check_csc(c)
    assert c.nnz == 7 * N ** 3 - 6 * N ** 2 == 14_581_760
    col = np.repeat(np.arange(c.n, dtype=np.int64), np.diff(c.colptr))
    row = c.rowidx.astype(np.int64)
    diag = row == col
    assert diag.sum() == c.n
    assert np.all((c.val[diag] >= 6 * 0.9) & (c.val[diag] <= 6 * 1.1))
    assert np.all((c.val[~diag] >= -1.1) & (c.val[~diag] <= -0.9))
    # A == A^T: the transposed entries, sorted the same way, are the same list
    t = np.lexsort((col, row))
    assert np.array_equal(row[t], col) and np.array_equal(col[t], row)
    assert np.array_equal(c.val[t], c.val)


def test_diag_poisson_parity_case():
    c = gen.diag_poisson(4096)
    check_csc(c)
    assert c.nnz == 20_340
    col = np.repeat(np.arange(c.n), np.diff(c.colptr))
    assert np.count_nonzero(c.rowidx == col) == c.n  # every column holds its diagonal
    assert np.all(np.abs(c.val) <= 1.0)


def test_batch_matrices():
    mats = gen.batch(count=6)
    assert len(mats) == 6
    for b, c in enumerate(mats):
        check_csc(c, np.float32)
        assert c.m == c.n and 1000 <= c.n <= 200_000
        if b % 2 == 0:
            assert c.degrees().min() >= 1  # Poisson degrees, at least one per column
    # the stream is drawn matrix by matrix: a shorter batch is a prefix
    again = gen.batch(count=2)
    assert all(np.array_equal(a.rowidx, b.rowidx) and np.array_equal(a.val, b.val) for a, b in zip(again, mats))


def test_to_csr_matches_a_dense_transpose():
    c = gen.zipf_columns(n=300, cap=40, seed=7)
    rowptr, colidx, val = c.to_csr()
    dense = np.zeros((c.m, c.n))
    for j in range(c.n):
        dense[c.rowidx[c.colptr[j]:c.colptr[j + 1]], j] = c.val[c.colptr[j]:c.colptr[j + 1]]
    back = np.zeros_like(dense)
    for i in range(c.m):
        seg = slice(rowptr[i], rowptr[i + 1])
        assert np.all(np.diff(colidx[seg]) > 0)
        back[i, colidx[seg]] = val[seg]
    assert np.array_equal(dense, back)
