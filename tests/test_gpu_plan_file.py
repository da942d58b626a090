"""Persistent plan files (fl_plan_save / fl_plan_load): a loaded plan equals
the saved one (info, exported reference layout, permutation, heavy band,
forms) and computes the same products; missing, truncated, corrupt and
invalid files are rejected with FL_ERR_IO / FL_ERR_ARG before any kernel
sees them."""
import numpy as np
import pytest

import oracle
from conftest import load_golden

pytestmark = pytest.mark.gpu

ERR_ARG, ERR_IO = -1, -7


def y_of(p, x, kernel=0):
    import torch

    xs = p.permute_x(torch.from_numpy(x).cuda())
    y = p.spmv(xs, kernel=kernel)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def matrices(gpu):
    from fastload_gb300 import gen

    g = load_golden("bus_i10")
    yield "bus_i10", g["m"], g["n"], g["cscptr"], g["cscrow"], g["cscval"]
    c = gen.diag_poisson(3000, seed=5)
    yield "poisson", c.m, c.n, c.colptr, c.rowidx, c.val
    c = gen.zipf_columns(40000, 1.8, 5000, seed=3)
    yield "zipf", c.m, c.n, c.colptr, c.rowidx, c.val
    # the automatic rule puts every column of a stencil in the band (x read
    # through the cache): the file records it and the load rebuilds it wide
    c = gen.laplacian7(16)
    yield "stencil", c.m, c.n, c.colptr, c.rowidx, c.val
    # empty columns and an empty matrix
    yield "empty_cols", 6, 5, np.array([0, 0, 2, 2, 5, 5]), np.array([1, 4, 0, 2, 5]), np.arange(1.0, 6.0)
    yield "empty", 4, 3, np.zeros(4, np.int64), np.zeros(0, np.int64), np.zeros(0)


@pytest.mark.parametrize("with_ref", [False, True])
@pytest.mark.parametrize("heavy", [-1, 0, 64])
def test_round_trip(gpu, tmp_path, with_ref, heavy):
    from fastload_gb300 import plan as P

    for name, m, n, cp, cr, cv in matrices(gpu):
        x = np.random.default_rng(1).uniform(-1, 1, n)
        band = heavy if heavy <= n else -1
        with gpu.Plan.from_csc(m, n, cp, cr, cv, with_reference_arrays=with_ref, heavy_band=band) as a:
            f = tmp_path / f"{name}.flplan"
            a.save(f)
            hdr = P.plan_file_header(f)
            assert (hdr["m"], hdr["n"], hdr["nnz"], hdr["tilenum"]) == (m, n, len(cr), a.info["tilenum"])
            sec = P.plan_file_sections(f)
            for k in ("perm", "sortnnz", "row", "val", "forms"):
                assert P.plan_file_hash(np.ascontiguousarray(sec[k]).tobytes()) == hdr["hashes"][k], (name, k)
            with gpu.Plan.load(f) as b:
                assert a.info == b.info, name
                if name == "stencil" and heavy == 0:
                    assert b.info["heavy_cols"] == n
                if with_ref:
                    sa, pa = a.export()
                    sb, pb = b.export()
                    np.testing.assert_array_equal(pa, pb)
                    for field in ("sortval", "sortrowidx", "tile_ptr", "tile_len", "tile_colidx", "tile_format",
                                  "countrow", "segmentoffset", "sortrowindex"):
                        np.testing.assert_array_equal(getattr(sa, field), getattr(sb, field), err_msg=field)
                if m and n:
                    yref = oracle.csc_spmv_dd(m, n, cp, cr, cv, x)
                    for kernel in (0, 2, 3) + ((1,) if with_ref else ()):
                        ya, yb = y_of(a, x, kernel), y_of(b, x, kernel)
                        if len(cr):
                            assert oracle.rel_errors(yb, yref)[0] <= 1e-12, (name, kernel)
                            assert oracle.rel_errors(ya, yb)[0] <= 1e-13, (name, kernel)
                b.check()


def test_forms_survive_round_trip(gpu, tmp_path):
    import torch

    from fastload_gb300 import gen

    c = gen.zipf_columns(30000, 1.8, 4000, seed=9)
    x = np.random.default_rng(2).uniform(-1, 1, c.n * 8)
    specs = [(gpu.VALUES_F32, gpu.BAND_ALL, False, {}), (gpu.VALUES_BF16X2, gpu.BAND_AUTO, False, {}),
             (gpu.VALUES_F32, gpu.BAND_NONE, True, {}), (gpu.VALUES_F64, 256, False, {}),
             (gpu.VALUES_F32, 2048, False, dict(light_item=512, heavy_loop=2, x_stage=1, unit_warps=8))]
    f = tmp_path / "forms.flplan"
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as a:
        ids = [a.add_form(v, band, y_f32=y32, **o) for v, band, y32, o in specs]
        a.save(f)
        with gpu.Plan.load(f) as b:
            for fid, (v, band, y32, o) in zip(ids, specs):
                assert a.form_info(fid) == b.form_info(fid)
                assert a.form_opts(fid) == b.form_opts(fid)
                for k, val in o.items():
                    assert b.form_opts(fid)[k] == val
                for k in (1, 8):
                    xs_a = a.permute_x_k(torch.from_numpy(x[:c.n * k]).cuda(), k=k, to_f32=v != 0)
                    xs_b = b.permute_x_k(torch.from_numpy(x[:c.n * k]).cuda(), k=k, to_f32=v != 0)
                    assert torch.equal(xs_a, xs_b)
                    ya = a.spmv_form(fid, xs_a, k=k).double().cpu().numpy()
                    yb = b.spmv_form(fid, xs_b, k=k).double().cpu().numpy()
                    tol = 1e-13 if v == 0 else 1e-6
                    assert oracle.rel_errors(ya, yb)[0] <= tol, (fid, k)
            b.check()


def test_missing_truncated_and_corrupt_files(gpu, tmp_path):
    from fastload_gb300 import FastLoadError, gen

    c = gen.diag_poisson(2000, seed=6)
    f = tmp_path / "p.flplan"
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as a:
        a.save(f)
        with pytest.raises(FastLoadError) as e:
            a.save(tmp_path)  # a directory
        assert e.value.code == ERR_IO
    raw = f.read_bytes()
    cases = {
        "missing": None,
        "truncated": raw[:-9],
        "header_only": raw[:128],
        "long": raw + b"\0" * 8,
        "magic": b"XXXXXXXX" + raw[8:],
        "header_bit": raw[:24] + bytes([raw[24] ^ 4]) + raw[25:],
        "value_bit": raw[:-100] + bytes([raw[-100] ^ 1]) + raw[-99:],
        "row_bit": raw[:128 + 8 * c.n + 3] + bytes([raw[128 + 8 * c.n + 3] ^ 1]) + raw[128 + 8 * c.n + 4:],
    }
    for name, data in cases.items():
        g = tmp_path / f"bad_{name}.flplan"
        if data is not None:
            g.write_bytes(data)
        with pytest.raises(FastLoadError) as e:
            gpu.Plan.load(g)
        assert e.value.code == ERR_IO, (name, e.value)


def test_invalid_content_with_valid_checksums(gpu, tmp_path):
    """Files whose checksums are right but whose content is not a FastLoad
    format (written by the test's own writer) are rejected by validation."""
    from fastload_gb300 import FastLoadError, gen
    from fastload_gb300 import plan as P

    c = gen.diag_poisson(1500, seed=7)
    f = tmp_path / "p.flplan"
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as a:
        a.save(f)
    hdr, sec = P.plan_file_header(f), P.plan_file_sections(f)

    def variant(name, code, **changes):
        s = {k: v.copy() for k, v in sec.items()}
        h = dict(hdr)
        for k, v in changes.items():
            if k in s:
                v(s[k])
            else:
                h[k] = v
        g = tmp_path / f"{name}.flplan"
        P.write_plan_file(g, h, s)
        with pytest.raises(FastLoadError) as e:
            gpu.Plan.load(g)
        assert e.value.code == code, (name, e.value)

    def bump_row(r):
        r[17] = c.m

    def neg_row(r):
        r[3] = -1

    def dup_perm(p):
        p[5] = p[6]

    def range_perm(p):
        p[0] = c.n

    def unsorted(s):
        s[0], s[-1] = s[-1], s[0]

    variant("row_range", ERR_ARG, row=bump_row)
    variant("row_negative", ERR_ARG, row=neg_row)
    variant("perm_dup", ERR_ARG, perm=dup_perm)
    variant("perm_range", ERR_ARG, perm=range_perm)
    variant("unsorted_counts", ERR_ARG, sortnnz=unsorted)
    variant("tilenum", ERR_IO, tilenum=hdr["tilenum"] + 1)
    variant("heavy_range", ERR_IO, heavy=c.n + 1)
    sec["forms"] = np.array([[7, 0, 0, 0, 0, 0, 0, 0]], np.int32)
    variant("form_type", ERR_ARG, nforms=1)
    # the valid file still loads after all of that
    with gpu.Plan.load(f) as b:
        assert b.info["nnz"] == c.nnz
