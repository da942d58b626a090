"""Comparators (naive CSC kernel, cuSPARSE CSR) against the compensated FP64
oracle on the golden cases: they are context lines in reports, so they must
compute the same product (normwise 1e-12; integer cases exactly)."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

INTEGER_CASES = {"bus_i10", "spmv9", "runs", "dups"}


def check(y, yref, integer, what):
    if integer:
        np.testing.assert_array_equal(y, yref, err_msg=what)
    else:
        assert oracle.rel_errors(y, yref)[0] <= 1e-12, what


@pytest.mark.parametrize("name", golden_names())
def test_comparators_match_oracle(gpu, name):
    import torch

    from fastload_gb300 import compare

    g = load_golden(name)
    m, n = g["m"], g["n"]
    if m == 0 or n == 0:
        pytest.skip("empty dimension")
    yref = oracle.csc_spmv_dd(m, n, g["cscptr"], g["cscrow"], g["cscval"], g["x"])
    dev = lambda a, t: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", t)  # noqa: E731
    cp, cr, cv = dev(g["cscptr"], torch.int32), dev(g["cscrow"], torch.int32), dev(g["cscval"], torch.float64)
    x = dev(g["x"], torch.float64)
    integer = name in INTEGER_CASES
    y = compare.csc_spmv_naive(m, cp, cr, cv, x)
    torch.cuda.synchronize()
    check(y.cpu().numpy(), yref, integer, name + "/naive")
    y2 = compare.csc_spmv_naive(m, cp, cr, cv, x, y=y.clone(), accumulate=True)
    torch.cuda.synchronize()
    check(y2.cpu().numpy(), 2 * yref, integer, name + "/naive+=")
    rp, ci, v = dev(g["rowptr"], torch.int32), dev(g["colidx"], torch.int32), dev(g["val"], torch.float64)
    for alg in (0, 1, 2):
        with compare.CuSparse(m, n, rp, ci, v, alg=alg) as cs:
            y = cs.spmv(x)
            y = cs.spmv(x, y=y)  # repeated calls on the prepared handle
            torch.cuda.synchronize()
            check(y.cpu().numpy(), yref, integer, f"{name}/cusparse{alg}")


def test_comparator_arguments(gpu):
    import torch

    from fastload_gb300 import FastLoadError, compare

    z = torch.zeros(4, dtype=torch.int32, device="cuda")
    with pytest.raises(FastLoadError):
        compare.CuSparse(0, 3, z, z, torch.zeros(4, dtype=torch.float64, device="cuda"))
    with pytest.raises(FastLoadError):
        compare.CuSparse(3, 3, z, z, torch.zeros(4, dtype=torch.float64, device="cuda"), alg=7)
