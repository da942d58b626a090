"""The sweep driver end to end on a small grid: every row complete, the
FastLoad plan agrees with the naive kernel, and the CSV keeps the
reference's data.py columns."""
import csv

import pytest

pytestmark = pytest.mark.gpu


def test_small_sweep(gpu, tmp_path):
    from fastload_gb300 import sweep

    out = tmp_path / "s.csv"
    rc = sweep.main(["--families", "random,poisson,banded", "--sizes", "1000,2000", "--sparsities", "50,95",
                     "--reps", "3", "--out", str(out)])
    assert rc == 0
    with open(out) as f:
        rows = list(csv.DictReader(f))
    assert len(rows) == 4 + 3 + 2
    for r in rows:
        assert r.keys() >= set(sweep.REF_HEADERS)
        assert int(r["nnz"]) > 0
        assert float(r["plan_kernel_ms"]) > 0 and float(r["Kernel_Time"]) > 0
        assert float(r["FastLoad_GPU_PASS_time"]) > 0
        assert float(r["rel_diff_vs_naive"]) <= 1e-12, r["case"]
        assert r["cusparse_ms"] != ""
