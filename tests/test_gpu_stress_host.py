"""Many host-buffer calls in a row on a matrix with a dense-column band and a
light part (the overlapped upload, the flag the light items wait for, the
programmatic dependent launches, the pipelined call's two staging slots):
every result within 1e-12 of the oracle, with a different x each call so a
stale slot, a missed wait or a reordered copy shows up as a wrong y."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-12


def test_many_host_calls(gpu):
    import torch

    from fastload_gb300 import gen

    c = gen.zipf_columns(1 << 17, 1.8, 20000, seed=7)
    rng = np.random.default_rng(3)
    nx = 6
    xs_true = [rng.uniform(-1, 1, c.n) for _ in range(nx)]
    refs = [oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, x) for x in xs_true]
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        assert 0 < p.info["heavy_cols"] < c.n and p.info["items"] > 0
        hx = [p.permute_x(torch.from_numpy(x).cuda()).cpu().pin_memory() for x in xs_true]
        # synchronous calls
        for i in range(150):
            y = p.spmv_host(hx[i % nx].numpy())
            e = oracle.rel_errors(y, refs[i % nx])[0]
            assert e <= FP64_TOL, ("sync", i, e)
        # pipelined calls: batches of eight in flight, each into its own buffer
        hy = [torch.empty(c.m, dtype=torch.float64).pin_memory() for _ in range(8)]
        for b in range(40):
            for j in range(8):
                hy[j].fill_(float("nan"))
            for j in range(8):
                p.spmv_host_async(hx[(b + j) % nx].numpy(), hy[j].numpy())
            torch.cuda.current_stream().synchronize()
            for j in range(8):
                e = oracle.rel_errors(hy[j].numpy(), refs[(b + j) % nx])[0]
                assert e <= FP64_TOL, ("async", b, j, e)
        p.check()
