"""Pipelined host-buffer SpMV (fl_plan_spmv_host_async): calls issued back to
back with distinct pinned x and y buffers, more calls in flight than the two
device staging slots, each result checked against the oracle; mixed with the
synchronous call; every layout kind (dense-column band with a light part,
band of every column, FastLoad stream only)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-12


def _cases():
    from fastload_gb300 import gen

    return [("dense columns", gen.zipf_columns(40000, 1.8, 5000, seed=3)),
            ("stencil", gen.laplacian7(24)),
            ("random rows", gen.diag_poisson(20000, seed=3))]


@pytest.mark.parametrize("case", [0, 1, 2])
def test_pipelined_host_calls(gpu, case):
    import torch

    name, c = _cases()[case]
    rng = np.random.default_rng(5)
    steps = 7
    xs_true = [rng.uniform(-1, 1, c.n) for _ in range(steps)]
    refs = [oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, x) for x in xs_true]
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        # x in the plan's sorted column order, in pinned host buffers
        hx_t = [p.permute_x(torch.from_numpy(x).cuda()).cpu().pin_memory() for x in xs_true]
        hy_t = [torch.full((c.m,), float("nan"), dtype=torch.float64).pin_memory() for _ in range(steps)]
        hx = [t.numpy() for t in hx_t]
        hy = [t.numpy() for t in hy_t]
        for i in range(steps):
            p.spmv_host_async(hx[i], hy[i])
            if i == 3:
                # a synchronous call in the middle of the pipeline
                ys = p.spmv_host(hx[0])
                assert oracle.rel_errors(ys, refs[0])[0] <= FP64_TOL, name
        torch.cuda.current_stream().synchronize()
        for i in range(steps):
            assert oracle.rel_errors(hy[i], refs[i])[0] <= FP64_TOL, (name, i)
        # the same host buffers again: results overwritten in place
        for i in range(steps):
            p.spmv_host_async(hx[steps - 1 - i], hy[i])
        torch.cuda.current_stream().synchronize()
        for i in range(steps):
            assert oracle.rel_errors(hy[i], refs[steps - 1 - i])[0] <= FP64_TOL, (name, i)
        p.check()


def test_pipelined_host_call_rejects_bad_buffers(gpu):
    from fastload_gb300 import gen

    c = gen.diag_poisson(1000, seed=1)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        with pytest.raises(ValueError):
            p.spmv_host_async(np.zeros(c.n, np.float32), np.zeros(c.m))
        with pytest.raises(ValueError):
            p.spmv_host_async(np.zeros(c.n - 1), np.zeros(c.m))
