"""The CPU oracle against the golden fixtures produced by the reference's own
CPU code (tests/golden/make_golden.py): every stage bit-exact."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden

LAYOUT_KEYS = ["tile_ptr", "tile_len", "tile_colidx", "tile_tall", "tile_format", "countrow", "segmentoffset",
               "sortrowindex", "sortrowidx", "sortval"]


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(name):
    g = load_golden(name)
    m, n = g["m"], g["n"]
    cp, cr, cv, cnt = oracle.csr2csc(m, n, g["rowptr"], g["colidx"], g["val"])
    np.testing.assert_array_equal(cp, g["cscptr"])
    np.testing.assert_array_equal(cr, g["cscrow"])
    np.testing.assert_array_equal(cv, g["cscval"])
    np.testing.assert_array_equal(cnt, g["nnzpercol"])
    perm, srow, sval, snnz, sx = oracle.col_sort(n, cnt, cp, cr, cv, g["x"])
    np.testing.assert_array_equal(perm, g["perm"])
    np.testing.assert_array_equal(snnz, g["sortnnz"])
    np.testing.assert_array_equal(snnz, g["ref_sortnnz"])  # same counts as the reference's std::sort
    np.testing.assert_array_equal(sx, g["sortx"])
    np.testing.assert_array_equal(srow, g["sortrowidx_tmp"])
    np.testing.assert_array_equal(sval, g["sortval_tmp"])
    lay = oracle.format_transform(n, g["nnz"], snnz, srow, sval)
    assert lay["tilenum"] == g["tilenum"]
    assert lay["segsum"] == g["segsum"]
    for k in LAYOUT_KEYS:
        np.testing.assert_array_equal(lay[k], g[k], err_msg=k)
    y = oracle.fastload_spmv(lay, sx, m)
    np.testing.assert_array_equal(y, g["y"])  # same tile-order summation as FastLoad_cpu


@pytest.mark.parametrize("name", golden_names())
def test_compensated_oracle_is_exactly_rounded(name):
    g = load_golden(name)
    y = oracle.csc_spmv_dd(g["m"], g["n"], g["cscptr"], g["cscrow"], g["cscval"], g["x"])
    ye = g["y_exact"]
    scale = max(float(np.max(np.abs(ye))) if ye.size else 0.0, 1e-300)
    assert float(np.max(np.abs(y - ye), initial=0.0)) <= 2e-16 * scale


def test_bus_pins_from_the_reference():
    """1138_bus as main.cu runs it: 139 tiles, 18 format-0 and 121 format-2
    tiles, and y equal to the CSC golden exactly (integer values)."""
    g = load_golden("bus_i10")
    assert g["tilenum"] == 139
    assert np.bincount(g["tile_format"], minlength=3).tolist() == [18, 0, 121]
    assert g["ref_pipeline_tilenum"] == 139
    yg = oracle.csc_spmv(g["n"], g["cscptr"], g["cscrow"], g["cscval"], g["x"], g["m"])
    yr = oracle.csr_spmv(g["m"], g["rowptr"], g["colidx"], g["val"], g["x"])
    np.testing.assert_array_equal(yg, yr)  # main.cu:122-132
    np.testing.assert_array_equal(g["y"], yg)  # FastLoad_CPU.h:33-44


def test_omp_tile_loop_matches_serial():
    g = load_golden("cfg1")
    lay = {k: g[k] for k in LAYOUT_KEYS}
    lay["tilenum"] = g["tilenum"]
    y1 = oracle.fastload_spmv(lay, g["sortx"], g["m"])
    y2, used = oracle.fastload_spmv(lay, g["sortx"], g["m"], threads=4)
    assert used >= 1
    np.testing.assert_allclose(y2, y1, rtol=0, atol=1e-13)
