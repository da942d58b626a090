"""Sweep driver host logic: the case grid of the reference's profiling
scripts and its random generator (test.cu:30-43 semantics)."""
import numpy as np

from fastload_gb300 import sweep


def test_grid_matches_reference_scripts():
    g = sweep.cases({"random"}, sweep.SIZES, sweep.SPARSITIES)
    assert len(g) == 70  # profiling/test.sh: 10 sparsities x 7 sizes
    names = [c[1] for c in g]
    assert len(set(names)) == len(names)
    assert "random_s95_n12000" in names
    allf = sweep.cases({"random", "poisson", "zipf", "laplacian", "banded", "block", "rowskew"}, (1000,), (50,))
    assert {c[0] for c in allf} == {"random", "poisson", "zipf", "laplacian", "banded", "block", "rowskew"}


def test_random_generator_density_and_order():
    for sp in (10, 50, 95):
        c = sweep.random_csc(800, sp, seed=3)
        dens = c.nnz / 800 ** 2
        assert abs(dens - (99 - sp) / 100) < 0.01, (sp, dens)
        for j in range(0, 800, 37):
            seg = c.rowidx[c.colptr[j]:c.colptr[j + 1]]
            assert np.all(np.diff(seg) > 0)
        assert c.val.min() >= 0 and c.val.max() < 1


def test_headers_keep_reference_columns():
    assert sweep.REF_HEADERS[:5] == ["sparsity", "matrix_size", "M", "N", "nnz"]
    assert len(sweep.REF_HEADERS) == 18
    assert sweep.main(["--list", "--families", "random", "--sizes", "1000", "--sparsities", "50"]) == 0
