"""MatrixMarket ingest on the GPU (fl_mtx_read / fl_mmio_allinone) against
the reference's reader: the committed fixtures (CSR from the reference's own
mmio_allinone) bit for bit, seeded random files of every kind against the
oracle's restatement, and 60k hard decimal spellings against correctly
rounded conversion (Python's float, which rounds as glibc's strtod does)."""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import ROOT
from mtx_cases import hard_decimals, write_random, write_value_file

pytestmark = pytest.mark.gpu

MTX_DIR = os.path.join(ROOT, "tests", "golden", "mtx")
NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(MTX_DIR, "*.mtx")))
ERR_ARG, ERR_IO = -1, -7


def golden(name):
    with np.load(os.path.join(MTX_DIR, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def gpu_csr(path):
    from fastload_gb300 import Mtx

    with Mtx.read(path) as mt:
        rp, ci, v = mt.to_torch()
        import torch

        torch.cuda.synchronize()
        return mt.info, rp.cpu().numpy(), ci.cpu().numpy(), v.cpu().numpy()


def assert_same(info, rp, ci, v, m, n, nnz, sym, grp, gci, gv):
    assert (info["m"], info["n"], info["nnz"], info["is_symmetric"]) == (m, n, nnz, sym)
    np.testing.assert_array_equal(rp, grp)
    np.testing.assert_array_equal(ci, gci)
    np.testing.assert_array_equal(np.asarray(v).view(np.uint64), np.asarray(gv).view(np.uint64))


@pytest.mark.parametrize("name", NAMES)
def test_fixtures_match_reference(gpu, name):
    g = golden(name)
    path = os.path.join(MTX_DIR, name + ".mtx")
    info, rp, ci, v = gpu_csr(path)
    assert_same(info, rp, ci, v, int(g["m"]), int(g["n"]), int(g["nnz"]), int(g["is_symmetric"]), g["rowptr"],
                g["colidx"], g["val"])
    # the host-array entry point returns the same
    m, n, nnz, sym, rp2, ci2, v2 = gpu.mmio_allinone(path)
    assert_same(dict(m=m, n=n, nnz=nnz, is_symmetric=sym), rp2, ci2, v2, int(g["m"]), int(g["n"]), int(g["nnz"]),
                int(g["is_symmetric"]), g["rowptr"], g["colidx"], g["val"])


def test_fixture_info(gpu):
    from fastload_gb300 import mtx

    info = gpu_csr(os.path.join(MTX_DIR, "complex_hermitian.mtx"))[0]
    assert (info["field"], info["symmetry"], info["nnz_file"]) == (mtx.COMPLEX, mtx.HERMITIAN, 4)
    info = gpu_csr(os.path.join(MTX_DIR, "real_skew.mtx"))[0]
    assert (info["symmetry"], info["is_symmetric"]) == (mtx.SKEW, 0)
    info = gpu_csr(os.path.join(MTX_DIR, "real_general.mtx"))[0]
    assert info["exact_path_values"] > 0  # the hard spellings need the big-integer path


@pytest.mark.parametrize("field,storage", [("real", "general"), ("real", "symmetric"), ("pattern", "general"),
                                           ("pattern", "symmetric"), ("integer", "symmetric"),
                                           ("complex", "general"), ("complex", "hermitian"),
                                           ("real", "skew-symmetric")])
def test_random_files_match_oracle(gpu, tmp_path, field, storage):
    p = tmp_path / "r.mtx"
    n = 5000
    write_random(p, n, n if storage != "general" else 3000, 120000, field, storage, seed=7)
    info, rp, ci, v = gpu_csr(p)
    assert_same(info, rp, ci, v, *oracle.mmio_read(p))


def test_hard_decimals_bit_exact(gpu, tmp_path):
    vals = hard_decimals(60000, seed=9)
    p = tmp_path / "v.mtx"
    write_value_file(p, vals)
    info, rp, ci, v = gpu_csr(p)
    expect = np.array([float(s) for s in vals])
    bad = np.nonzero(v.view(np.uint64) != expect.view(np.uint64))[0]
    assert bad.size == 0, [(vals[i][:60], v[i], expect[i]) for i in bad[:5]]
    assert info["exact_path_values"] > 1000


def test_many_entries_and_segments(gpu, tmp_path):
    """A few million entries: token indexing across chunk boundaries."""
    p = tmp_path / "big.mtx"
    write_random(p, 200000, 150000, 2_000_000, "real", "general", seed=11)
    info, rp, ci, v = gpu_csr(p)
    assert_same(info, rp, ci, v, *oracle.mmio_read(p))


def test_plan_from_mtx(gpu, tmp_path):
    import torch

    p = tmp_path / "s.mtx"
    write_random(p, 4000, 4000, 30000, "real", "symmetric", seed=12)
    m, n, nnz, sym, rp, ci, v = oracle.mmio_read(p)
    cp, cr, cv, _ = oracle.csr2csc(m, n, rp, ci, v)
    x = np.random.default_rng(0).uniform(-1, 1, n)
    yref = oracle.csc_spmv_dd(m, n, cp, cr, cv, x)
    with gpu.Plan.from_mtx(p, with_reference_arrays=True) as plan:
        assert plan.info["nnz"] == nnz
        y = plan.spmv(plan.permute_x(torch.from_numpy(x).cuda()))
        torch.cuda.synchronize()
        assert oracle.rel_errors(y.cpu().numpy(), yref)[0] <= 1e-12
        with gpu.Plan.from_csr(m, n, rp, ci, v, with_reference_arrays=True) as q:
            a, pa = plan.export()
            b, pb = q.export()
            np.testing.assert_array_equal(pa, pb)
            np.testing.assert_array_equal(a.sortval.view(np.uint64), b.sortval.view(np.uint64))
            np.testing.assert_array_equal(a.sortrowidx, b.sortrowidx)


def test_bad_files_rejected(gpu, tmp_path):
    from fastload_gb300 import FastLoadError, Mtx

    cases = {
        "banner": ("%%MatrixMarket matrix coordinate real\n1 1 1\n1 1 1\n", ERR_ARG),
        "no_banner": ("1 1 1\n1 1 1\n", ERR_ARG),
        "array": ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", ERR_ARG),
        "row_range": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", ERR_ARG),
        "col_zero": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 0 1.0\n", ERR_ARG),
        "short": ("%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1.0\n2 2 2.0\n", ERR_ARG),
        "index_token": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1.5 1.0\n", ERR_ARG),
        "value_token": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1.2.3\n", ERR_ARG),
        "value_exp": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1e\n", ERR_ARG),
        "hex": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 0x1.8p3\n", ERR_ARG),
        "nan_payload": ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 nan(12)\n", ERR_ARG),
        "int_value": ("%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 2.5\n", ERR_ARG),
        "int_overflow": ("%%MatrixMarket matrix coordinate integer general\n2 2 1\n1 1 2147483648\n", ERR_ARG),
        "size": ("%%MatrixMarket matrix coordinate real general\n2 x 1\n1 1 1\n", ERR_ARG),
        "sym_rect": ("%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 3 1.0\n", ERR_ARG),
        "empty_file": ("", ERR_IO),
    }
    for name, (text, code) in cases.items():
        p = tmp_path / f"{name}.mtx"
        p.write_text(text)
        with pytest.raises(FastLoadError) as e:
            Mtx.read(p)
        assert e.value.code == code, (name, e.value)
    with pytest.raises(FastLoadError) as e:
        Mtx.read(tmp_path / "missing.mtx")
    assert e.value.code == ERR_IO
    # the context is still usable
    info = gpu_csr(os.path.join(MTX_DIR, "real_symmetric.mtx"))[0]
    assert info["nnz"] == 13
