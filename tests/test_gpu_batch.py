"""Batches: many matrices of uneven size in one persistent launch, direct and
replayed through a captured CUDA graph, against the compensated FP64 oracle.

Tolerance (normwise, per matrix): FP64 values 1e-12; FP32 and BF16 hi+lo
values 1e-6, with FP64 y and with FP32 accumulation into FP32 y alike."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _mats(count=20, seed=21):
    from fastload_gb300 import gen

    ms = gen.batch(count, seed=seed, nmin=64, nmax=4000, dtype=np.float64)
    ms.append(gen.from_csr_lists(5, 7, [], x=np.ones(7)))  # an empty matrix in the stack
    return ms


@pytest.mark.parametrize("vtype,y_f32,tol", [(0, False, 1e-12), (1, False, 1e-6), (1, True, 1e-6), (2, False, 1e-6)])
def test_batch_matches_oracle(gpu, vtype, y_f32, tol):
    import torch

    mats = _mats()
    plans = [gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val, heavy_band=-1) for c in mats]
    with gpu.Batch(plans, value_type=vtype, y_f32=y_f32) as b:
        for p in plans:
            p.close()  # the batch keeps its own copy
        assert b.count == len(mats) and b.nnz == sum(c.nnz for c in mats)
        x = torch.from_numpy(np.concatenate([c.x for c in mats])).cuda()
        xs = b.permute_x(x)
        y1 = b.spmv(xs).double().cpu().numpy()
        y2 = b.spmv_graph(xs).double().cpu().numpy()
        y3 = b.spmv_graph(xs).double().cpu().numpy()  # replay
        yo = torch.empty(b.m, dtype=torch.float32 if y_f32 else torch.float64, device="cuda")
        y4 = b.spmv_graph(xs, yo).double().cpu().numpy()  # new y pointer: recapture
        for yy in (y1, y2, y3, y4):
            for i, c in enumerate(mats):
                ref = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
                got = yy[b.m_off[i]:b.m_off[i + 1]]
                if c.nnz == 0:
                    assert not got.any()
                    continue
                nw, mx = oracle.rel_errors(got, ref)
                assert nw <= tol, (i, nw, mx)


def test_batch_rejects_bad_arguments(gpu):
    from fastload_gb300 import _lib

    lib = _lib.load()
    import ctypes as C

    h = C.c_void_p()
    assert lib.fl_batch_create(C.byref(h), 1, None, 1, 1) == -1
    mats = _mats(2)
    plans = [gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) for c in mats]
    with pytest.raises(gpu.FastLoadError):
        gpu.Batch(plans, value_type=2, y_f32=True)


@pytest.mark.parametrize("empty_rows", [False, True])
def test_batch_overwrites_stale_y(gpu, empty_rows):
    """Rows are owned by one lane and stored, not accumulated: whatever y held
    before (here NaN) is replaced, including rows without nonzeros."""
    import torch

    from fastload_gb300 import gen

    mats = [gen.diag_poisson(n, seed=n) for n in (300, 1000, 77)]
    if empty_rows:
        mats.append(gen.from_csr_lists(6, 4, [(0, 0, 1.5), (2, 1, -2.0), (2, 3, 3.0), (5, 2, 4.0)],
                                       x=np.arange(4.0)))  # rows 1, 3, 4 empty
    plans = [gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) for c in mats]
    with gpu.Batch(plans, value_type=0, y_f32=False) as b:
        x = torch.from_numpy(np.concatenate([c.x for c in mats])).cuda()
        xs = b.permute_x(x)
        for run in (b.spmv, b.spmv_graph):
            y = torch.full((b.m,), float("nan"), dtype=torch.float64, device="cuda")
            yy = run(xs, y).cpu().numpy()
            assert np.isfinite(yy).all()
            for i, c in enumerate(mats):
                ref = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
                assert oracle.rel_errors(yy[b.m_off[i]:b.m_off[i + 1]], ref)[0] <= 1e-12
    for p in plans:
        p.close()


def test_batch_full_size_256_matrices(gpu):
    """The batched workload at its stated size: 256 seeded matrices, n
    log-uniform in [1e3, 2e5], mean degree U[4, 32], half Poisson and half
    Zipf(1.5) column degrees (186M nonzeros in all), FP32 values with FP32
    accumulation into FP32 y, one launch direct and replayed from the
    captured graph; every matrix within 1e-6 of the compensated FP64 oracle."""
    import torch

    from fastload_gb300 import gen

    mats = gen.batch(256, seed=3, dtype=np.float64)
    assert len(mats) == 256
    plans = [gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) for c in mats]
    with gpu.Batch(plans, value_type=gpu.VALUES_F32, y_f32=True) as b:
        for p in plans:
            p.close()
        assert b.nnz == sum(c.nnz for c in mats) and b.nnz > 1.5e8
        x = torch.from_numpy(np.concatenate([c.x for c in mats])).cuda()
        xs = b.permute_x(x)
        ys = [b.spmv(xs).double().cpu().numpy()]
        y = torch.empty(b.m, dtype=torch.float32, device="cuda")
        for _ in range(2):  # capture, then replay
            ys.append(b.spmv_graph(xs, y).double().cpu().numpy())
        worst = 0.0
        for i, c in enumerate(mats):
            ref = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
            for yy in ys:
                nw, mx = oracle.rel_errors(yy[b.m_off[i]:b.m_off[i + 1]], ref)
                assert nw <= 1e-6, (i, c.m, c.nnz, nw, mx)
                worst = max(worst, nw)
        print(f"batch of {len(mats)} matrices, {b.nnz} nonzeros: worst normwise error {worst:.2e}")
