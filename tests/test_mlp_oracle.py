"""The CPU reference of the tuner network checks itself by finite
differences (float64) -- so it can serve as the oracle of the CUDA
gradients in tests/test_gpu_tuner.py."""
import numpy as np

from oracle import mlp


def test_numpy_mlp_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    shape = (5, 7, 6, 3)
    n = 5 * 7 + 7 + 7 * 6 + 6 + 6 * 3 + 3
    p = rng.normal(0, 0.5, n)
    X = rng.normal(size=(11, 5))
    T = rng.normal(size=(11, 3))
    M = (rng.random((11, 3)) > 0.2).astype(float)
    loss, g = mlp.loss_grad(p, shape, X, T, M)
    eps = 1e-6
    fd = np.empty(n)
    for i in range(n):
        q = p.copy()
        q[i] += eps
        lp, _ = mlp.loss_grad(q, shape, X, T, M)
        q[i] -= 2 * eps
        lm, _ = mlp.loss_grad(q, shape, X, T, M)
        fd[i] = (lp - lm) / (2 * eps)
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-7)


def test_tuner_targets_and_regret():
    """Targets are log2(t / t_best) over the timed variants; untimed (NaN)
    variants are masked out; regret is against the best timed variant and
    the default variant is the library's automatic choice."""
    from fastload_gb300 import tuner

    V = len(tuner.VARIANTS)
    t = np.full((2, V), np.nan)
    t[0, :4] = [2.0, 1.0, 4.0, 1.5]
    t[1, :4] = [1.0, 1.1, 1.2, 1.3]
    tg, m = tuner.targets(t), tuner.mask_of(t)
    np.testing.assert_allclose(tg[0, :4], np.log2(t[0, :4] / 1.0))
    assert np.all(tg[:, 4:] == 0) and np.all(m[:, 4:] == 0) and np.all(m[:, :4] == 1)
    ev = tuner.evaluate(np.array([1, 0]), t)
    assert ev["mean_regret"] == 0.0 and ev["frac_within_10pct"] == 1.0
    assert tuner.DEFAULT == 0 and tuner.PLAIN == 1
    assert ev["speedup_vs_auto_rule"] == (2.0 + 1.0) / (1.0 + 1.0)


def test_tuner_variant_table():
    """The search space comes from the library (fl_tuner_variants): every
    knob the tuner chooses -- heavy band, light item size, heavy loop, x
    staging, units per warp, BF16 hi+lo storage -- takes more than one value,
    and BF16 variants are offered to FP32 callers only."""
    from fastload_gb300 import tuner

    T = tuner.TABLE
    assert len(T) == len(set(tuner.VARIANTS)) >= 60
    for k in ("heavy_band", "light_item", "heavy_loop", "x_stage", "unit_warps", "value_type"):
        assert len({o[k] for o in T}) >= 2, k
    a64, a32 = tuner.allowed(0), tuner.allowed(1)
    assert a64.sum() * 2 == a32.sum() == len(T)
    assert all(o["value_type"] == tuner.TUNE_REQUESTED for o, ok in zip(T, a64) if ok)


def test_tuner_specs_cover_the_families_and_ranges():
    from fastload_gb300 import tuner

    rng = np.random.default_rng(5)
    specs = [tuner.sample_spec(rng, i) for i in range(200)]
    assert {s["family"] for s in specs} == set(tuner.FAMILIES)
    for s in specs[:40]:
        assert tuner.N_RANGE[0] * 0.99 <= s["n"] <= tuner.N_RANGE[1] * 1.01
        d = tuner.degrees(s)
        assert d.shape == (s["n"],) and d.min() >= 0 and d.sum() <= tuner.NNZ_RANGE[1] * 1.06
        if s["family"] == "banded":
            assert d.max() <= max(1, int(s["param"]))


def test_committed_model_and_data_match_the_variant_table():
    """The committed tuner model (the library's format, which
    fl_plan_add_tuned_form reads) and autotuner data were made over the
    library's current variant table: magic, shape, the table itself, and a
    file size that matches the shape.  Read without a GPU."""
    import os

    from fastload_gb300 import tuner

    raw = open(tuner.MODEL, "rb").read()
    assert raw[:8] == b"FLTUNER1"
    n_in, h1, h2, n_out, nv = (int(v) for v in np.frombuffer(raw, "<i4", 5, 8))
    assert (n_in, n_out, nv) == (24, len(tuner.TABLE), len(tuner.TABLE))
    n_params = n_in * h1 + h1 + h1 * h2 + h2 + h2 * n_out + n_out
    assert len(raw) == 40 + 4 * (2 * n_in + n_params) + 32 * nv
    opts = np.frombuffer(raw, "<i4", 8 * nv, len(raw) - 32 * nv).reshape(nv, 8)
    fields = ("value_type", "heavy_band", "y_f32", "light_item", "heavy_loop", "x_stage", "unit_warps", "reserved")
    assert [dict(zip(fields, map(int, r))) for r in opts] == tuner.TABLE
    data = os.path.join(os.path.dirname(tuner.MODEL), "cfg5_autotune.npz")
    with np.load(data) as z:
        assert tuple(str(v) for v in z["variants"]) == tuner.VARIANTS
        T = z["T"]
        assert T.shape == (2200, len(tuner.TABLE))
        assert np.all(np.isfinite(T) | np.isnan(T)) and np.nanmin(T) > 0
