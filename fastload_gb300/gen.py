"""Seeded synthetic sparse matrices for the FastLoad workloads.

The reference is evaluated on SuiteSparse matrices that are not available
here; these generators stand in with the shapes, sizes and value
distributions of the benchmark configurations:

* ``diag_poisson``  -- square n, each column its diagonal plus Poisson(lam)
  extra nonzeros at distinct uniform rows; values and x U[-1, 1].
* ``zipf_columns``  -- square n, column degrees Zipf(s) capped, distinct
  uniform rows; values N(0, 1), x U[-1, 1].
* ``laplacian7``    -- 7-point 3D Laplacian on an N^3 grid with +-jitter on
  every value and symmetric off-diagonal perturbation.
* ``batch``         -- many independent matrices, log-uniform n, mean
  degree U[4, 32], half Poisson and half Zipf(1.5) column degrees.

All return CSC with rows ascending inside each column (the layout
src/csr2csc_cuda.h produces) as a ``CSC`` record; numpy PCG64 seeds make
them reproducible.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CSC:
    m: int
    n: int
    colptr: np.ndarray  # int32, n+1
    rowidx: np.ndarray  # int32, nnz
    val: np.ndarray     # float64 (or float32), nnz
    x: np.ndarray       # float64 (or float32), n

    @property
    def nnz(self) -> int:
        return int(self.rowidx.size)

    def degrees(self) -> np.ndarray:
        return np.diff(self.colptr).astype(np.int32)

    def to_csr(self):
        """(rowptr, colidx, val) of the same matrix, columns ascending per row."""
        col = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.colptr))
        order = np.argsort(self.rowidx, kind="stable")
        rowptr = np.zeros(self.m + 1, np.int64)
        np.cumsum(np.bincount(self.rowidx, minlength=self.m), out=rowptr[1:])
        return rowptr.astype(np.int32), col[order].astype(np.int32), self.val[order]


def _sorted_unique(a: np.ndarray) -> np.ndarray:
    """np.unique for int64 keys via sort + adjacent compare (much faster
    than np.unique on tens of millions of keys)."""
    a = np.sort(a)
    if a.size < 2:
        return a
    keep = np.empty(a.size, bool)
    keep[0] = True
    np.not_equal(a[1:], a[:-1], out=keep[1:])
    return a[keep]


def _distinct_rows(rng: np.random.Generator, m: int, deg: np.ndarray, forced_rows=None):
    """For column c draw deg[c] distinct rows uniformly from [0, m) (plus the
    forced row of c when given).  Returns sorted int64 keys col*m + row."""
    n = deg.size
    deg = np.minimum(deg.astype(np.int64), m)
    # dense columns (a quarter of the rows or more) are drawn exactly, the
    # rest by vectorised rejection of duplicates
    dense = np.flatnonzero(deg * 4 >= m) if m > 0 else np.zeros(0, np.int64)
    dense_keys = []
    for c in dense:
        rows = rng.choice(m, size=int(deg[c]), replace=False).astype(np.int64)
        if forced_rows is not None and forced_rows[c] not in rows:
            rows[0] = forced_rows[c]
        dense_keys.append(c * m + rows)
    if dense.size:
        deg = deg.copy()
        deg[dense] = 0
    target = deg.copy()
    if forced_rows is not None:
        forced_rows = np.asarray(forced_rows, np.int64).copy()
    cols = np.repeat(np.arange(n, dtype=np.int64), deg)
    keys = cols * m + rng.integers(0, m, size=cols.size)
    if forced_rows is not None:
        sparse = np.ones(n, bool)
        sparse[dense] = False
        keys = np.concatenate([keys, np.flatnonzero(sparse).astype(np.int64) * m + forced_rows[sparse]])
        target = np.where(sparse, np.minimum(target + 1, m), 0)
    keys = _sorted_unique(keys)
    for _ in range(256):
        cnt = np.bincount(keys // m, minlength=n)
        deficit = target - cnt
        if not deficit.any():
            if dense_keys:
                keys = np.sort(np.concatenate([keys] + dense_keys))
            return keys
        # over-full columns (forced row drawn twice can't happen: unique) are
        # impossible; draw more for the short ones
        dcols = np.repeat(np.arange(n, dtype=np.int64), np.maximum(deficit, 0))
        extra = _sorted_unique(dcols * m + rng.integers(0, m, size=dcols.size))
        pos = np.searchsorted(keys, extra)
        present = (pos < keys.size) & (keys[np.minimum(pos, keys.size - 1)] == extra)
        extra = extra[~present]
        if extra.size:
            # keep only as many new rows per column as the deficit allows
            ecols = extra // m
            first = np.searchsorted(ecols, ecols, side="left")
            rank = np.arange(extra.size) - first
            extra = extra[rank < deficit[ecols]]
            keys = np.concatenate([keys, extra])
            keys.sort(kind="stable")
    raise RuntimeError("distinct row sampling did not converge")


def _csc_from_keys(m: int, n: int, keys: np.ndarray, val: np.ndarray, x: np.ndarray) -> CSC:
    cols = keys // m
    rows = (keys - cols * m).astype(np.int32)
    colptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(cols, minlength=n), out=colptr[1:])
    return CSC(m, n, colptr.astype(np.int32), rows, val, x)


def diag_poisson(n: int = 4096, lam: float = 4.0, seed: int = 1) -> CSC:
    """Square n; diagonal plus Poisson(lam) distinct uniform rows per column."""
    rng = np.random.default_rng(seed)
    extra = np.minimum(rng.poisson(lam, size=n), n - 1)
    keys = _distinct_rows(rng, n, extra, forced_rows=np.arange(n, dtype=np.int64))
    val = rng.uniform(-1.0, 1.0, size=keys.size)
    x = rng.uniform(-1.0, 1.0, size=n)
    return _csc_from_keys(n, n, keys, val, x)


def zipf_degrees(rng: np.random.Generator, n: int, s: float, cap: int) -> np.ndarray:
    return np.minimum(rng.zipf(s, size=n), cap).astype(np.int64)


def zipf_columns(n: int = 1 << 20, s: float = 1.8, cap: int = 50000, seed: int = 2, m: int | None = None,
                 dtype=np.float64) -> CSC:
    """Column degrees Zipf(s) capped at `cap`; distinct uniform rows."""
    m = n if m is None else m
    rng = np.random.default_rng(seed)
    deg = zipf_degrees(rng, n, s, min(cap, m))
    keys = _distinct_rows(rng, m, deg)
    val = rng.standard_normal(size=keys.size).astype(dtype)
    x = rng.uniform(-1.0, 1.0, size=n).astype(dtype)
    return _csc_from_keys(m, n, keys, val, x)


def laplacian7(N: int = 128, jitter: float = 0.1, seed: int = 4, dtype=np.float64) -> CSC:
    """7-point Laplacian on an N^3 grid (index i + N j + N^2 k), diagonal
    6(1+u), off-diagonals -(1+u) with one u per edge so A is symmetric."""
    rng = np.random.default_rng(seed)
    n = N * N * N
    c = np.arange(n, dtype=np.int64)
    i, j, k = c % N, (c // N) % N, c // (N * N)
    diag = 6.0 * (1.0 + rng.uniform(-jitter, jitter, size=n))
    # edge (a, a+d) perturbation, indexed by a, for d = 1, N, N^2
    steps = [(1, i), (N, j), (N * N, k)]
    edge = {d: -(1.0 + rng.uniform(-jitter, jitter, size=n)) for d, _ in steps}
    offsets = []  # (offset, valid mask over columns, values)
    for d, coord in reversed(steps):  # -N^2, -N, -1
        ok = coord > 0
        v = np.zeros(n)
        v[ok] = edge[d][c[ok] - d]
        offsets.append((-d, ok, v))
    offsets.append((0, np.ones(n, bool), diag))
    for d, coord in steps:  # +1, +N, +N^2
        ok = coord < N - 1
        v = np.zeros(n)
        v[ok] = edge[d][c[ok]]
        offsets.append((d, ok, v))
    cnt = sum(ok.astype(np.int64) for _, ok, _ in offsets)
    colptr = np.zeros(n + 1, np.int64)
    np.cumsum(cnt, out=colptr[1:])
    nnz = int(colptr[-1])
    rows = np.empty(nnz, np.int32)
    vals = np.empty(nnz, dtype)
    filled = np.zeros(n, np.int64)
    for off, ok, v in offsets:
        cc = c[ok]
        pos = colptr[cc] + filled[cc]
        rows[pos] = (cc + off).astype(np.int32)
        vals[pos] = v[ok]
        filled[cc] += 1
    x = rng.uniform(-1.0, 1.0, size=n).astype(dtype)
    return CSC(n, n, colptr.astype(np.int32), rows, vals, x)


def _zipf_cap_for_mean(s: float, mean: float, limit: int) -> int:
    """Smallest cap with E[min(Zipf(s), cap)] >= mean (cap <= limit)."""
    k = np.arange(1, limit + 1, dtype=np.float64)
    p = k ** (-s)
    p /= p.sum()
    tail = np.cumsum(p[::-1])[::-1]  # P(Z >= k)
    # E[min(Z, c)] = sum_{k=1}^{c} P(Z >= k)
    e = np.cumsum(tail)
    idx = int(np.searchsorted(e, mean))
    return int(min(idx + 1, limit))


def batch(count: int = 256, seed: int = 3, nmin: float = 1e3, nmax: float = 2e5, dtype=np.float32) -> list[CSC]:
    """Independent square matrices: n log-uniform, mean degree U[4, 32],
    even index -> Poisson(mean) degrees (min 1), odd -> Zipf(1.5) capped so
    its mean matches."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(count):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        mean = rng.uniform(4.0, 32.0)
        if b % 2 == 0:
            deg = np.maximum(rng.poisson(mean, size=n), 1)
        else:
            cap = _zipf_cap_for_mean(1.5, mean, min(n, 1 << 20))
            deg = zipf_degrees(rng, n, 1.5, cap)
        keys = _distinct_rows(rng, n, np.minimum(deg, n))
        val = rng.standard_normal(size=keys.size).astype(dtype)
        x = rng.uniform(-1.0, 1.0, size=n).astype(dtype)
        out.append(_csc_from_keys(n, n, keys, val, x))
    return out


def from_csr_lists(m: int, n: int, entries, x=None) -> CSC:
    """Small hand-made matrices: entries = [(row, col, val), ...]."""
    e = sorted(entries, key=lambda t: (t[1], t[0]))
    colptr = np.zeros(n + 1, np.int64)
    for _, c, _ in e:
        colptr[c + 1] += 1
    colptr = np.cumsum(colptr)
    rows = np.array([r for r, _, _ in e], np.int32)
    vals = np.array([v for _, _, v in e], np.float64)
    xx = np.ones(n) if x is None else np.asarray(x, np.float64)
    return CSC(m, n, colptr.astype(np.int32), rows, vals, xx)
