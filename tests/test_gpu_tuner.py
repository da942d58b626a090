"""The tuner's GPU pieces: the network's CUDA forward/backward against the CPU
reference (oracle/mlp.py), training, the matrix generator and the feature
extractor; and, when the committed autotuner data is present, the trained
network's held-out regret and its gain over the method without it."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import mlp as mlp_ref

pytestmark = pytest.mark.gpu

DATA = os.path.join(ROOT, "fastload_gb300", "tuner_data", "cfg5_autotune.npz")


def test_mlp_forward_and_gradient_match_cpu_reference(gpu):
    from fastload_gb300 import tuner

    rng = np.random.default_rng(3)
    net = tuner.Network(seed=7)
    p = net.params()
    K = net.shape[3]
    X = rng.normal(size=(97, 24)).astype(np.float32)
    T = rng.normal(size=(97, K)).astype(np.float32)
    M = (rng.random((97, K)) > 0.1).astype(np.float32)
    Y = net.forward_raw(X)
    Yr, _ = mlp_ref.forward(p, net.shape, X)
    np.testing.assert_allclose(Y, Yr, rtol=1e-4, atol=1e-4)
    loss, g = net.grad_raw(X, T, M)
    lr, gr = mlp_ref.loss_grad(p, net.shape, X, T, M)
    assert abs(loss - lr) <= 1e-4 * max(1.0, abs(lr))
    err = np.abs(g - gr) / (np.abs(gr).max() + 1e-12)
    assert err.max() <= 1e-4, err.max()
    net.close()


def test_mlp_training_reduces_loss(gpu):
    from fastload_gb300 import tuner

    rng = np.random.default_rng(4)
    X = rng.normal(size=(256, 24)).astype(np.float32)
    W = rng.normal(size=(24, 6))
    times = np.exp(np.tanh(X @ W) + 1.0)  # a learnable best-variant structure
    net = tuner.Network(seed=2, n_out=6)
    losses = net.fit(X, times, epochs=400, lr=3e-3)
    assert losses[-1] < 0.25 * losses[0]
    ev = tuner.evaluate(net.predict(X), times)
    assert ev["mean_regret"] < 0.2
    net.close()


@pytest.mark.parametrize("family,param", [(0, 0.0), (2, 40.0), (3, 64.0), (4, 3.0)])
def test_generator_rows(gpu, family, param):
    import torch

    from fastload_gb300 import _lib

    n = m = 5000
    rng = np.random.default_rng(family)
    d = rng.integers(1, 30, n)
    if family in (2, 3):
        d = np.minimum(d, int(param))
    colptr = np.concatenate([[0], np.cumsum(d)]).astype(np.int32)
    nnz = int(colptr[-1])
    cp = torch.from_numpy(colptr).cuda()
    rows = torch.empty(nnz, dtype=torch.int32, device="cuda")
    vals = torch.empty(nnz, dtype=torch.float64, device="cuda")
    lib = _lib.load()
    assert lib.fl_gen_fill(family, m, n, C.c_void_p(cp.data_ptr()), C.c_void_p(rows.data_ptr()),
                           C.c_void_p(vals.data_ptr()), param, C.c_ulonglong(99), None) == 0
    r = rows.cpu().numpy()
    v = vals.cpu().numpy()
    assert r.min() >= 0 and r.max() < m and np.all(np.abs(v) <= 1.0)
    for c in range(0, n, 97):
        seg = r[colptr[c]:colptr[c + 1]]
        assert np.all(np.diff(seg) >= 0)
        if family == 2:
            centre = c * m // n
            assert np.all(np.abs(seg - centre) <= param / 2 + 1)
        if family == 3:
            blk = (c * m // n) // int(param)
            assert np.all(seg // int(param) == blk)
    # deterministic in the seed
    rows2 = torch.empty_like(rows)
    lib.fl_gen_fill(family, m, n, C.c_void_p(cp.data_ptr()), C.c_void_p(rows2.data_ptr()),
                    C.c_void_p(vals.data_ptr()), param, C.c_ulonglong(99), None)
    assert torch.equal(rows, rows2)


def test_features_match_numpy(gpu):
    from fastload_gb300 import gen, tuner

    c = gen.zipf_columns(20000, 1.8, 5000, seed=8)
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val, heavy_band=-1) as p:
        f = tuner.features(p, 1)
    deg = np.diff(c.colptr).astype(float)
    assert abs(f[0] - np.log10(c.n)) < 1e-5 and abs(f[2] - np.log10(c.nnz)) < 1e-5
    assert abs(f[4] - deg.std() / deg.mean()) < 1e-3
    hist = np.bincount(np.minimum(np.floor(np.log2(deg[deg > 0])).astype(int), 10), minlength=11) / c.n
    np.testing.assert_allclose(f[7:18], hist, atol=1e-6)
    sd = np.sort(deg)
    for i, b in enumerate((2048, 8192, 24576)):
        assert abs(f[18 + i] - sd[-min(b, c.n):].sum() / c.nnz) < 1e-5
    col = np.repeat(np.arange(c.n), np.diff(c.colptr))
    band = np.abs(c.rowidx / c.m - col / c.n).mean()
    assert abs(f[21] - band) < 1e-4
    rc = np.bincount(c.rowidx, minlength=c.m).astype(float)
    assert abs(f[22] - rc.std() / rc.mean()) < 1e-3
    assert f[23] == 1.0


def _data():
    """The committed autotuner data, when it was collected over the
    library's current variant table."""
    from fastload_gb300 import tuner

    if not os.path.exists(DATA):
        return None
    with np.load(DATA) as z:
        data = {k: z[k] for k in z.files}
    if tuple(str(v) for v in data["variants"]) != tuner.VARIANTS:
        return None
    return data


MODEL = os.path.join(ROOT, "fastload_gb300", "tuner_data", "model.fltuner")


def test_trained_tuner_heldout_regret(gpu):
    """Trained on 2000 matrices of the committed autotuner data, evaluated on
    200 held-out ones: mean regret against the exhaustive autotuner over the
    whole variant table at most 10%, and at least as fast in total as the
    method without the tuner (the library's automatic choices)."""
    from fastload_gb300 import tuner

    data = _data()
    if data is None:
        pytest.skip("autotuner data for the current variant table not collected")
    res = tuner.train_and_evaluate(data, n_train=2000, epochs=3000, seed=1)
    h = res["heldout"]
    assert h["matrices"] >= 150 and h["variants"] == len(tuner.VARIANTS)
    assert h["mean_regret"] <= 0.10, h
    assert h["speedup_vs_auto_rule"] >= 1.0, h


def test_tuned_form_through_the_c_abi_follows_the_committed_model(gpu):
    """fl_plan_add_tuned_form (Plan.add_tuned_form) regenerates held-out
    matrices of the autotuner data from their specs and picks, through the C
    ABI, the variant the committed model predicts from the stored features
    (the Python choice, tuner.choose, agrees); the tuned form computes the
    product within its value type's tolerance."""
    import json

    import torch

    import oracle
    from fastload_gb300 import tuner

    data = _data()
    if data is None or not os.path.exists(MODEL):
        pytest.skip("trained model for the current variant table not committed")
    X, T, metas = data["X"], data["T"], [json.loads(m) for m in data["meta"]]
    net = tuner.load_model(MODEL)
    expect = net.predict(X, np.isfinite(T))
    net.close()
    picked, bf16 = 0, 0
    for i in range(2000, len(metas)):
        spec = metas[i]
        if spec["nnz"] > 3_000_000:
            continue
        plan, nnz, x = tuner.make_plan(spec)
        try:
            fid, variant = plan.add_tuned_form(spec["values"])
            assert variant == tuner.VARIANTS[int(expect[i])], (i, variant)
            assert tuner.choose(plan, spec["values"], MODEL)[1] == variant
            vt = plan.form_info(fid)["value_type"]
            assert vt == spec["values"] or (spec["values"] == 1 and vt == 2)
            bf16 += vt == 2
            xs = plan.permute_x_k(x, k=1, to_f32=vt != 0)
            y = plan.spmv_form(fid, xs)
            y0 = plan.spmv(plan.permute_x(x))
            torch.cuda.synchronize()
            rel = oracle.rel_errors(y.double().cpu().numpy(), y0.cpu().numpy())[0]
            assert rel <= (1e-12 if vt == 0 else 1e-6), (i, rel)
            plan.check()
        finally:
            plan.close()
        picked += 1
        if picked == 16:
            break
    assert picked >= 8


def test_tuned_form_rejects_bad_model_files(gpu, tmp_path):
    from fastload_gb300 import FastLoadError, gen

    c = gen.diag_poisson(3000, seed=4)
    bad = tmp_path / "bad.fltuner"
    bad.write_bytes(b"FLTUNER1" + np.array([24, 64, 64, 5, 5, 0, 0, 0], "<i4").tobytes())
    with gpu.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        for path, code in ((tmp_path / "missing.fltuner", -7), (bad, -1)):
            with pytest.raises(FastLoadError) as e:
                p.add_tuned_form(1, model=path)
            assert e.value.code == code, e.value
        trunc = tmp_path / "trunc.fltuner"
        if os.path.exists(MODEL):
            trunc.write_bytes(open(MODEL, "rb").read()[:-7])
            with pytest.raises(FastLoadError) as e:
                p.add_tuned_form(1, model=trunc)
            assert e.value.code == -7
        with pytest.raises(FastLoadError):
            p.add_tuned_form(2, model=bad)  # BF16 is not a caller's type
