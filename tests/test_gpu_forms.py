"""Storage / right-hand-side forms against the compensated FP64 oracle.

Tolerances (normwise ||y - y*||_2 / ||y*||_2, y* = exactly rounded A x on the
original FP64 values and x):
  FP64 values               1e-12
  FP32 values, FP32 x       1e-6   (the FP32-path target of the workload)
  BF16 hi+lo values, FP32 x 1e-6   (hi = bf16(v) plus a 16-bit correction:
                                    23 significant bits, within 2^-23 + 2^-24
                                    of each value once decoded)
Integer-valued matrices (values and x small integers) are exact in every
form."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 1e-6, 2: 1e-6}
INTEGER_CASES = {"bus_i10", "spmv9", "runs", "dups"}


def run_form(gpu, p, fid, vtype, x, k):
    import torch

    xs = p.permute_x_k(torch.from_numpy(np.ascontiguousarray(x.reshape(-1))).cuda(), k=k, to_f32=vtype != 0)
    y = p.spmv_form(fid, xs, k=k)
    torch.cuda.synchronize()
    return y.cpu().numpy().reshape(-1, k) if k > 1 else y.cpu().numpy()


def check(y, yref, vtype, integer, what):
    if integer:
        np.testing.assert_array_equal(y, yref, err_msg=what)
        return
    nw, mx = oracle.rel_errors(np.asarray(y).reshape(-1), np.asarray(yref).reshape(-1))
    assert nw <= TOL[vtype], (what, nw, mx)


@pytest.mark.parametrize("name", golden_names())
def test_forms_match_oracle(gpu, name):
    g = load_golden(name)
    m, n = g["m"], g["n"]
    rng = np.random.default_rng(7)
    integer = name in INTEGER_CASES
    x8 = (np.arange(n * 8) % 10).astype(float) if integer else rng.uniform(-1, 1, n * 8)
    yref1 = oracle.csc_spmv_dd(m, n, g["cscptr"], g["cscrow"], g["cscval"], g["x"])
    yref8 = oracle.csc_spmv_dd(m, n, g["cscptr"], g["cscrow"], g["cscval"], x8, k=8)
    with gpu.Plan.from_csr(m, n, g["rowptr"], g["colidx"], g["val"]) as p:
        forced = min(n, 64) & ~1
        bands = [gpu.BAND_NONE, gpu.BAND_AUTO, gpu.BAND_ALL] + ([forced] if forced > 0 else [])
        for vtype in (gpu.VALUES_F64, gpu.VALUES_F32, gpu.VALUES_BF16X2):
            for band in bands:
                fid = p.add_form(vtype, band)
                what = f"{name}/v{vtype}/band{band}"
                check(run_form(gpu, p, fid, vtype, g["x"], 1), yref1, vtype, integer, what + "/k1")
                check(run_form(gpu, p, fid, vtype, x8, 8), yref8, vtype, integer, what + "/k8")
        p.check()


def test_form_fp32_y(gpu):
    """FP32 values with FP32 accumulation into an FP32 y."""
    import torch

    g = load_golden("cfg1")
    with gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"]) as p:
        fid = p.add_form(gpu.VALUES_F32, gpu.BAND_ALL, y_f32=True)
        assert p.form_info(fid)["y_f32"] == 1
        xs = p.permute_x_k(torch.from_numpy(g["x"]).cuda(), k=1, to_f32=True)
        y = p.spmv_form(fid, xs, y_f32=True)
        assert y.dtype == torch.float32
        nw, mx = oracle.rel_errors(y.cpu().numpy().astype(np.float64), g["y_exact"])
        assert nw <= 1e-6, nw


def test_form_accumulate(gpu):
    import torch

    g = load_golden("zipf_small")
    with gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"]) as p:
        for band in (gpu.BAND_NONE, gpu.BAND_ALL, 512):
            fid = p.add_form(gpu.VALUES_F64, band)
            xs = p.permute_x_k(torch.from_numpy(g["x"]).cuda(), k=1)
            y = p.spmv_form(fid, xs)
            p.spmv_form(fid, xs, y=y, accumulate=True)
            nw, _ = oracle.rel_errors(y.cpu().numpy() / 2, g["y_exact"])
            assert nw <= 1e-12, (band, nw)


def test_form_rejects_bad_arguments(gpu):
    import torch

    g = load_golden("cfg1")
    with gpu.Plan.from_csr(g["m"], g["n"], g["rowptr"], g["colidx"], g["val"]) as p:
        with pytest.raises(gpu.FastLoadError):
            p.add_form(7, gpu.BAND_AUTO)
        with pytest.raises(gpu.FastLoadError):
            p.add_form(gpu.VALUES_BF16X2, gpu.BAND_AUTO, y_f32=True)
        fid = p.add_form(gpu.VALUES_F32, gpu.BAND_NONE)
        xs = torch.zeros(g["n"] * 3, dtype=torch.float32, device="cuda")
        with pytest.raises(gpu.FastLoadError):
            p.spmv_form(fid, xs, k=3)


@pytest.mark.parametrize("vtype", [1, 2])
def test_full_size_laplacian_forms(gpu, vtype):
    """The 128^3 Laplacian (14.6M nonzeros) in FP32 / BF16 hi+lo, k = 1 and 8,
    with and without the all-column row slices."""
    from fastload_gb300 import gen

    c = gen.laplacian7(128, seed=4)
    rng = np.random.default_rng(11)
    x8 = rng.uniform(-1, 1, c.n * 8)
    yref1 = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
    yref8 = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, x8, k=8)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        for band in (gpu.BAND_NONE, gpu.BAND_ALL):
            fid = p.add_form(vtype, band)
            check(run_form(gpu, p, fid, vtype, c.x, 1), yref1, vtype, False, f"lap/v{vtype}/b{band}/k1")
            check(run_form(gpu, p, fid, vtype, x8, 8), yref8, vtype, False, f"lap/v{vtype}/b{band}/k8")
        p.check()


def test_full_size_zipf_auto_band(gpu):
    """The 2^20-column Zipf(1.8) matrix (27M nonzeros) in FP32 and BF16
    hi+lo with the automatic heavy band."""
    from fastload_gb300 import gen

    c = gen.zipf_columns(1 << 20, 1.8, 50000, seed=2)
    yref = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        for vtype in (gpu.VALUES_F32, gpu.VALUES_BF16X2):
            fid = p.add_form(vtype, gpu.BAND_AUTO)
            assert p.form_info(fid)["heavy_cols"] > 0
            check(run_form(gpu, p, fid, vtype, c.x, 1), yref, vtype, False, f"zipf/v{vtype}")
        p.check()


def test_convert_values_matches_oracle(gpu):
    """The device's storage conversion equals the oracle's restatement bit
    for bit: BF16 hi+lo words and FP32 values, over many magnitudes, ties,
    zeros, subnormals and the BF16 overflow threshold."""
    rng = np.random.default_rng(5)
    v = rng.standard_normal(200_000) * np.exp(rng.uniform(-80, 80, 200_000))
    ties = 1.0 + np.arange(1, 256) * 2.0 ** -8  # every tie of the BF16 rounding in [1, 2)
    special = np.array([0.0, -0.0, 1e-40, -1e-40, 2.0 ** -101, 2.0 ** -99, 3.38e38, 3.4e38, -3.4e38, 1e300,
                        np.inf, -np.inf])
    v = np.concatenate([v, ties, -ties, special])
    w = gpu.convert_values(v, gpu.VALUES_BF16X2).cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(w, oracle.bf16x2_split(v))
    f = gpu.convert_values(v, gpu.VALUES_F32).cpu().numpy()
    with np.errstate(over="ignore"):
        np.testing.assert_array_equal(f, v.astype(np.float32))


@pytest.mark.parametrize("vtype", [0, 1, 2])
def test_heavy_band_paths_agree(gpu, vtype):
    """The three heavy-band paths on one matrix: a band whose x fits shared
    memory beside the per-warp cp.async rings (16,384 columns), a band too
    wide for the rings but not for shared memory (the register-pipelined
    loop: 20,000 FP64 / 47,000 FP32 columns), and every column (x read from
    global memory)."""
    from fastload_gb300 import gen

    c = gen.zipf_columns(60000, 1.5, 3000, seed=17)
    yref = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
    wide = 20000 if vtype == 0 else 47000
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        for band in (16384, wide, gpu.BAND_ALL):
            fid = p.add_form(vtype, band)
            info = p.form_info(fid)
            assert info["heavy_cols"] == (c.n if band == gpu.BAND_ALL else band)
            check(run_form(gpu, p, fid, vtype, c.x, 1), yref, vtype, False, f"v{vtype}/band{band}")
        p.check()


@pytest.mark.parametrize("vtype", [0, 1, 2])
def test_form_options_match_oracle(gpu, vtype):
    """Every build / launch option of a form (light item size, heavy loop,
    x staging, units per warp; fl_form_opts) computes the same product
    within the form's tolerance, including the shared-memory ring with a
    unit boundary inside a pack and the register loop with x read through
    the cache.  Launch options changed in place take effect."""
    from fastload_gb300 import gen

    c = gen.zipf_columns(70000, 1.6, 5000, seed=23)
    yref = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        for band in (gpu.BAND_AUTO, 4096, gpu.BAND_ALL):
            for light in (0, 128, 1024):
                for heavy, xst in ((1, 0), (2, 0), (2, 1)):
                    for units in (0, 1, 16):
                        fid = p.add_form(vtype, band, light_item=light, heavy_loop=heavy, x_stage=xst,
                                         unit_warps=units)
                        o = p.form_opts(fid)
                        assert (o["light_item"], o["heavy_loop"], o["x_stage"], o["unit_warps"]) == \
                            (light, heavy, xst, units)
                        check(run_form(gpu, p, fid, vtype, c.x, 1), yref, vtype, False,
                              f"v{vtype}/b{band}/l{light}/h{heavy}/x{xst}/u{units}")
        fid = p.add_form(vtype, 4096)
        for heavy, xst in ((1, 0), (2, 0), (2, 1), (0, 0)):
            p.set_form_launch(fid, heavy, xst)
            assert (p.form_opts(fid)["heavy_loop"], p.form_opts(fid)["x_stage"]) == (heavy, xst)
            check(run_form(gpu, p, fid, vtype, c.x, 1), yref, vtype, False, f"launch h{heavy}/x{xst}")
        for bad in (dict(light_item=100), dict(light_item=9000), dict(heavy_loop=3), dict(x_stage=2),
                    dict(unit_warps=65)):
            with pytest.raises(gpu.FastLoadError):
                p.add_form(vtype, gpu.BAND_AUTO, **bad)
        p.check()
