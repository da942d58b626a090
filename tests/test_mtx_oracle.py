"""MatrixMarket reader of the oracle (fo_mmio_read) against the reference's
own mmio_allinone: the committed fixtures it produced (tests/golden/mtx),
and, where the reference was compiled here (oracle/_ref), seeded random files
and the hard decimal spellings."""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import ROOT
from mtx_cases import hard_decimals, write_random, write_value_file

MTX_DIR = os.path.join(ROOT, "tests", "golden", "mtx")
NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(MTX_DIR, "*.mtx")))


def golden(name):
    with np.load(os.path.join(MTX_DIR, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def same_csr(a, g):
    m, n, nnz, sym, rp, ci, v = a
    assert (m, n, nnz, sym) == (int(g["m"]), int(g["n"]), int(g["nnz"]), int(g["is_symmetric"]))
    np.testing.assert_array_equal(rp, g["rowptr"])
    np.testing.assert_array_equal(ci, g["colidx"])
    np.testing.assert_array_equal(np.asarray(v).view(np.uint64), np.asarray(g["val"]).view(np.uint64))


def test_fixture_set_is_complete():
    assert len(NAMES) >= 10
    for n in NAMES:
        assert os.path.exists(os.path.join(MTX_DIR, n + ".npz"))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_fixtures(name):
    same_csr(oracle.mmio_read(os.path.join(MTX_DIR, name + ".mtx")), golden(name))


def _ref():
    try:
        from oracle import ref

        ref.lib()
        return ref
    except Exception:
        return None


@pytest.mark.parametrize("field,storage", [("real", "general"), ("real", "symmetric"), ("pattern", "symmetric"),
                                           ("integer", "general"), ("complex", "hermitian"),
                                           ("real", "skew-symmetric")])
def test_oracle_matches_reference_random(tmp_path, field, storage):
    ref = _ref()
    if ref is None:
        pytest.skip("reference reader not compiled here")
    p = tmp_path / "r.mtx"
    write_random(p, 300, 300 if storage != "general" else 200, 4000, field, storage, seed=3)
    m, n, nnz, sym, rp, ci, v = ref.mmio_read(str(p))
    same_csr(oracle.mmio_read(p), dict(m=m, n=n, nnz=nnz, is_symmetric=sym, rowptr=rp, colidx=ci, val=v))


def test_oracle_hard_decimals_match_python_and_reference(tmp_path):
    vals = hard_decimals(3000, seed=2)
    p = tmp_path / "v.mtx"
    write_value_file(p, vals)
    m, n, nnz, sym, rp, ci, v = oracle.mmio_read(p)
    expect = np.array([float(s) for s in vals])
    np.testing.assert_array_equal(v.view(np.uint64), expect.view(np.uint64))
    ref = _ref()
    if ref is not None:
        np.testing.assert_array_equal(ref.mmio_read(str(p))[6].view(np.uint64), expect.view(np.uint64))


def test_oracle_rejects_bad_files(tmp_path):
    bad = {
        "banner": "%%MatrixMarket matrix coordinate real\n1 1 1\n1 1 1\n",
        "array": "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
        "range": "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n",
        "short": "%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1.0\n2 2 2.0\n",
        "token": "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 x 1.0\n",
        "sym_rect": "%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 3 1.0\n",
    }
    for name, text in bad.items():
        p = tmp_path / f"{name}.mtx"
        p.write_text(text)
        with pytest.raises(ValueError):
            oracle.mmio_read(p)
    with pytest.raises(ValueError):
        oracle.mmio_read(tmp_path / "missing.mtx")
