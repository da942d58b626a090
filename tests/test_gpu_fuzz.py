"""Seeded fuzz over matrix shapes: tall and wide rectangles, empty rows and
columns, a dense row, a band of dense columns, skewed rows, single rows and
columns, short-and-wide matrices whose long slices are cut across work units,
a medium Zipf matrix.  Each goes through the plan's automatic layout (y = A x,
y += A x, the stream kernel), the FP64 form with every heavy-band choice
(none, 2,048 columns, all; k = 1 and, for all, k = 8), and the host-buffer
calls (synchronous and pipelined).  FP64 results within 1e-12 normwise of
the compensated oracle."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-12


def _matrix(kind, seed):
    from fastload_gb300 import gen

    rng = np.random.default_rng(seed)
    if kind == "medium_zipf":
        return gen.zipf_columns(60000, 1.6, 8000, seed=seed)
    shapes = {"rect_tall": (3000, 500), "rect_wide": (400, 5000), "empty_rows_cols": (3000, 3000),
              "dense_row": (4000, 4000), "dense_cols": (6000, 6000), "skewed_rows": (5000, 5000),
              "one_col": (5000, 1), "one_row": (1, 5000), "cut_slices": (200, 40000)}
    m, n = shapes[kind]
    cols, rows = [], []
    if kind == "cut_slices":
        deg = rng.poisson(60, n)
    elif kind == "one_row":
        deg = (rng.random(n) < 0.7).astype(np.int64)
    else:
        deg = rng.poisson(6 if m > 1000 else 3, n)
    if kind == "empty_rows_cols":
        deg[rng.random(n) < 0.3] = 0
    if kind == "dense_cols":
        deg[rng.choice(n, 80, replace=False)] = 2000  # enough dense columns for a band
    deg = np.minimum(deg, m)
    for c in np.nonzero(deg)[0]:
        if kind == "skewed_rows":
            p = 1.0 / np.arange(1, m + 1) ** 1.2
            r = rng.choice(m, deg[c], replace=False, p=p / p.sum())
        elif kind == "empty_rows_cols":
            r = rng.choice(m // 2, min(deg[c], m // 2), replace=False) * 2  # odd rows stay empty
        else:
            r = rng.choice(m, deg[c], replace=False)
        rows.append(r)
        cols.append(np.full(len(r), c))
    if kind == "dense_row":
        extra = np.nonzero(rng.random(n) < 0.8)[0]
        rows.append(np.full(len(extra), 17))
        cols.append(extra)
    r = np.concatenate(rows).astype(np.int64)
    c = np.concatenate(cols).astype(np.int64)
    keys = np.unique(c * m + r)
    return gen._csc_from_keys(m, n, keys, rng.standard_normal(keys.size), rng.uniform(-1, 1, n))


KINDS = ["rect_tall", "rect_wide", "empty_rows_cols", "dense_row", "dense_cols", "skewed_rows", "one_col",
         "one_row", "cut_slices", "medium_zipf"]


@pytest.mark.parametrize("kind", KINDS)
def test_fuzz_every_path(gpu, kind):
    import torch

    c = _matrix(kind, seed=KINDS.index(kind) + 40)
    assert c.nnz > 0
    ydd = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
    ok = lambda y, what: _check(y, ydd, f"{kind}/{what}")  # noqa: E731
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        xs = p.permute_x(torch.from_numpy(c.x).cuda())
        y = torch.full((c.m,), float("nan"), dtype=torch.float64, device="cuda")
        p.spmv(xs, y)
        ok(y.cpu().numpy(), "auto")
        p.spmv(xs, y, accumulate=True)
        ok(y.cpu().numpy() / 2, "accumulate")
        ok(p.spmv(xs, kernel=gpu.KERNEL_STREAM).cpu().numpy(), "stream")
        hx = xs.cpu().numpy()
        ok(p.spmv_host(hx), "host")
        hx_p = torch.from_numpy(hx).pin_memory()
        hy_p = [torch.full((c.m,), float("nan"), dtype=torch.float64).pin_memory() for _ in range(3)]
        for t in hy_p:
            p.spmv_host_async(hx_p.numpy(), t.numpy())
        torch.cuda.current_stream().synchronize()
        for i, t in enumerate(hy_p):
            ok(t.numpy(), f"host_async{i}")
        bands = [("none", gpu.BAND_NONE), ("all", gpu.BAND_ALL)] + ([("2048", 2048)] if c.n >= 4096 else [])
        for name, band in bands:
            fid = p.add_form(gpu.VALUES_F64, band)
            yf = torch.full((c.m,), float("nan"), dtype=torch.float64, device="cuda")
            p.spmv_form(fid, xs, yf)
            ok(yf.cpu().numpy(), f"form_{name}")
            if name == "all":
                k = 8
                xk = np.random.default_rng(1).uniform(-1, 1, c.n * k)
                ydk = np.asarray(oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, xk, k=k)).reshape(-1)
                yk = p.spmv_form(fid, p.permute_x_k(torch.from_numpy(xk).cuda(), k=k), k=k)
                e = oracle.rel_errors(yk.cpu().numpy(), ydk)[0]
                assert e <= FP64_TOL, (kind, "form_all_k8", e)
        p.check()


def _check(y, ydd, what):
    assert np.all(np.isfinite(y)), what
    e = oracle.rel_errors(y, ydd)[0]
    assert e <= FP64_TOL, (what, e)
