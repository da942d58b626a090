"""Learned tuner: picks a matrix's complete form configuration from 24
plan features with a small MLP trained on the project's own exhaustive
autotuner timings.

The search space is the library's variant table (fl_tuner_variants, one
network output each), for the caller's value type and, for callers asking
for FP32 values, the BF16 hi+lo storage (both meet the 1e-6 error bar):

    default   the library's automatic choices (the method without the tuner)
    none      the FastLoad tile stream alone, light items auto / 512 / 1024
    all       every column as row slices (rows owned by one lane), heavy
              units 4 or 2 per warp
    band      the 8,192 / 24,576 / 49,152 densest columns as row slices
              x light items auto / 512 / 1024
              x heavy loop: shared-memory ring, registers with x staged in
                shared memory, registers with x read through the cache

The training set: seeded matrices of five families (uniform rows, Zipf
column degrees, banded, block-diagonal, row-skewed) generated on the GPU
(fl_gen_fill), n log-uniform in [1e4, 4e6], nnz log-uniform in [1e5, 6e7],
FP64 or FP32 values.  Every variant the matrix's caller may use is built
and timed with calls back to back (the steady state of repeated SpMVs):
on one plan for matrices whose streams can stay in L2 between calls,
alternating between two copies of the plan for larger ones, so that their
calls find the matrix out of L2.  The
network (24 -> 64 -> 64 -> one output per variant, ReLU) regresses
log2(t_variant / t_best), the variants a matrix may not use masked out, and
is trained on the GPU by the library's own forward/backward/Adam kernels
(fl_mlp_*); the autotuner's measurements are what regret is measured
against.  The trained network is stored in the library's model format, which
fl_plan_add_tuned_form reads, so C callers get the tuned form through the C
ABI.

    python -m fastload_gb300.tuner collect --count 2200 --out data.npz
    python -m fastload_gb300.tuner train --data data.npz
    python -m fastload_gb300.tuner evaluate --data data.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

import numpy as np

from ._lib import FastLoadArgumentError, FormOptsC, check, load

FAMILIES = ("uniform", "zipf", "banded", "blockdiag", "rowskew")
N_FEATURES = 24
N_RANGE = (1e4, 4e6)
NNZ_RANGE = (1e5, 6e7)
TUNE_REQUESTED = -1  # FL_TUNE_REQUESTED: the caller's value type
_OPT_FIELDS = tuple(k for k, _ in FormOptsC._fields_)


def variant_table() -> list[dict]:
    """The library's variant table (fl_tuner_variants), as option dicts."""
    n = load().fl_tuner_variants(None, 0)
    arr = (FormOptsC * n)()
    load().fl_tuner_variants(arr, n)
    return [{k: int(getattr(o, k)) for k in _OPT_FIELDS} for o in arr]


def variant_name(o: dict) -> str:
    parts = ["req" if o["value_type"] == TUNE_REQUESTED else "bf16x2",
             "band=" + {0: "auto", -1: "none", -2: "all"}.get(o["heavy_band"], str(o["heavy_band"]))]
    if o["light_item"]:
        parts.append(f"light={o['light_item']}")
    if o["heavy_loop"]:
        parts.append({1: "ring", 2: "regs"}[o["heavy_loop"]])
    if o["x_stage"]:
        parts.append("xglobal")
    if o["unit_warps"]:
        parts.append(f"units={o['unit_warps']}")
    return "|".join(parts)


TABLE = variant_table()
VARIANTS = tuple(variant_name(o) for o in TABLE)
DEFAULT = VARIANTS.index("req|band=auto")   # the library's automatic choices
PLAIN = VARIANTS.index("req|band=none")     # the FastLoad tile stream alone


def allowed(value_type: int) -> np.ndarray:
    """Variants a caller asking for value_type (0 FP64, 1 FP32) may get: its
    own type, plus BF16 hi+lo storage for FP32 callers."""
    return np.array([o["value_type"] == TUNE_REQUESTED or (o["value_type"] == 2 and value_type == 1)
                     for o in TABLE])


def resolved(o: dict, value_type: int) -> dict:
    """A variant's options for a caller of value_type."""
    r = dict(o)
    if r["value_type"] == TUNE_REQUESTED:
        r["value_type"] = int(value_type)
    return r


# ------------------------------------------------------------ generation --
def sample_spec(rng: np.random.Generator, index: int) -> dict:
    family = FAMILIES[index % len(FAMILIES)]
    n = int(round(np.exp(rng.uniform(np.log(N_RANGE[0]), np.log(N_RANGE[1])))))
    nnz = float(np.exp(rng.uniform(np.log(NNZ_RANGE[0]), np.log(NNZ_RANGE[1]))))
    spec = {"family": family, "n": n, "m": n, "nnz_target": nnz, "seed": int(rng.integers(1 << 62)),
            "values": int(rng.integers(2))}  # 0 FP64 values, 1 FP32 values
    if family == "zipf":
        spec["param"] = float(rng.uniform(1.5, 2.2))
    elif family == "banded":
        spec["param"] = float(np.exp(rng.uniform(0.0, np.log(512.0))))
    elif family == "blockdiag":
        spec["param"] = float(np.exp(rng.uniform(np.log(32.0), np.log(1024.0))))
    elif family == "rowskew":
        spec["param"] = float(rng.uniform(1.5, 4.0))
    else:
        spec["param"] = 0.0
    return spec


def degrees(spec: dict) -> np.ndarray:
    """Per-column nonzero counts of a spec (host, numpy)."""
    rng = np.random.default_rng(spec["seed"])
    n, m = spec["n"], spec["m"]
    mean = min(max(spec["nnz_target"] / n, 1.0), float(m))
    fam = spec["family"]
    if fam == "zipf":
        z = np.minimum(rng.zipf(spec["param"], size=n), m).astype(np.float64)
        d = np.maximum(1, np.round(z * (mean / z.mean())))
    else:
        d = rng.poisson(mean, size=n).astype(np.float64)
        if fam == "banded":
            d = np.minimum(d, max(1, int(spec["param"])))
        elif fam == "blockdiag":
            d = np.minimum(d, max(1, int(spec["param"])))
    d = np.minimum(d, m).astype(np.int64)
    cap = int(NNZ_RANGE[1] * 1.05)
    if d.sum() > cap:
        d = np.floor(d * (cap / d.sum())).astype(np.int64)
    return d


def make_plan(spec: dict, heavy_band: int = -1, copies: int = 1):
    """Generates the spec's matrix on the GPU and builds its plan.
    Returns (plan, nnz, device x); with copies > 1 the plan is a list of
    that many plans of the same matrix."""
    import torch

    from .plan import Plan

    d = degrees(spec)
    colptr = np.zeros(spec["n"] + 1, np.int64)
    np.cumsum(d, out=colptr[1:])
    nnz = int(colptr[-1])
    cp = torch.from_numpy(colptr.astype(np.int32)).cuda()
    rows = torch.empty(max(nnz, 1), dtype=torch.int32, device="cuda")
    vals = torch.empty(max(nnz, 1), dtype=torch.float64, device="cuda")
    check(load().fl_gen_fill(FAMILIES.index(spec["family"]), spec["m"], spec["n"], C.c_void_p(cp.data_ptr()),
                             C.c_void_p(rows.data_ptr()), C.c_void_p(vals.data_ptr()), float(spec["param"]),
                             C.c_ulonglong(spec["seed"] & ((1 << 64) - 1)), None))
    torch.cuda.synchronize()
    plans = [Plan.from_csc(spec["m"], spec["n"], cp, rows[:nnz], vals[:nnz], heavy_band=heavy_band)
             for _ in range(copies)]
    g = torch.Generator(device="cuda")
    g.manual_seed(spec["seed"] & 0x7FFFFFFF)
    x = torch.rand(spec["n"], dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    del rows, vals, cp
    return (plans[0] if copies == 1 else plans), nnz, x


def is_large(nnz: int, value_type: int) -> bool:
    """Streams too large to stay in L2 between one SpMV and the next in
    practice (COLD_BYTES)."""
    return nnz * ((8 if value_type == 0 else 4) + 4) > COLD_BYTES


def features(plan, value_type: int) -> np.ndarray:
    out = np.zeros(N_FEATURES, np.float32)
    check(load().fl_plan_features(plan._h, int(value_type), out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


# ------------------------------------------------------------- autotune --
def _time_calls(fns, reps: int) -> float:
    """Mean device ms of one call over reps calls back to back, cycling
    through fns (one callable per copy of the matrix: with two copies each
    call finds its matrix evicted from L2 by the other's call), after two
    untimed rounds; a device sleep ahead of the start event lets the host
    enqueue the calls first, so small matrices are not timed at the host's
    pace."""
    import torch

    for f in fns * 2:
        f()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda._sleep(600_000)
    a.record()
    for i in range(reps):
        fns[i % len(fns)]()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / reps


# Streams above this many bytes do not stay in L2 (129 MB) from one SpMV to
# the next in practice (their own size, or the rest of an application's
# working set, evicts them): such matrices are timed alternating between two
# copies of their plan; smaller ones back to back on one, as they run when
# repeated.
COLD_BYTES = 48 << 20


def autotune(plans, x, value_type: int, reps: int = 8) -> np.ndarray:
    """Exhaustive over the variant table: every variant value_type's caller
    may use is built as a form of the plan (variants that differ only in
    launch options share one build) and timed.  plans: a plan, or a list of
    plans of the same matrix whose calls alternate (large matrices).
    Returns ms per variant, NaN where the variant is not allowed."""
    import torch

    plans = plans if isinstance(plans, list) else [plans]
    p0 = plans[0]
    times = np.full(len(TABLE), np.nan)
    ok = allowed(value_type)
    xs = {}
    y = torch.empty(p0.m, dtype=torch.float64, device="cuda")
    groups: dict = {}
    for i, o in enumerate(TABLE):
        if ok[i]:
            r = resolved(o, value_type)
            key = (r["value_type"], r["heavy_band"], r["light_item"], r["unit_warps"])
            groups.setdefault(key, []).append((i, r["heavy_loop"], r["x_stage"]))
    for (vt, band, light, units), members in groups.items():
        fids = [p.add_form(vt, band, light_item=light, unit_warps=units) for p in plans]
        f32 = vt != 0
        if f32 not in xs:
            xs[f32] = p0.permute_x_k(x, k=1, to_f32=f32)
        fns = [lambda p=p, f=f: p.spmv_form(f, xs[f32], y) for p, f in zip(plans, fids)]
        for i, heavy, xst in members:
            for p, f in zip(plans, fids):
                p.set_form_launch(f, heavy, xst)
            times[i] = _time_calls(fns, reps)
    for p in plans:
        p.check()
    return times


def collect(count: int, seed: int = 5, out: str | None = None, log_every: int = 50) -> dict:
    rng = np.random.default_rng(seed)
    X, T, meta = [], [], []
    t0 = time.time()

    def pack():
        return {"X": np.array(X, np.float32).reshape(-1, N_FEATURES),
                "T": np.array(T, np.float64).reshape(-1, len(TABLE)),
                "meta": np.array([json.dumps(m) for m in meta]), "variants": np.array(VARIANTS)}

    # one untimed round on a small matrix first: the first launches of each
    # kernel pay one-time costs (module loading, shared-memory opt-in)
    warm, _, xw = make_plan({"family": "uniform", "n": 20000, "m": 20000, "nnz_target": 2e5, "seed": 1,
                             "values": 1, "param": 0.0}, copies=2)
    try:
        autotune(warm, xw, 1, reps=2)
    finally:
        for p in warm:
            p.close()
    for i in range(count):
        spec = sample_spec(rng, i)
        copies = 2 if is_large(int(degrees(spec).sum()), spec["values"]) else 1
        plans, nnz, x = make_plan(spec, copies=copies)
        plans = plans if isinstance(plans, list) else [plans]
        try:
            f = features(plans[0], spec["values"])
            t = autotune(plans, x, spec["values"])
        finally:
            for p in plans:
                p.close()
        X.append(f)
        T.append(t)
        meta.append(dict(spec, nnz=nnz))
        if log_every and (i + 1) % log_every == 0:
            print(f"[tuner] {i + 1}/{count} matrices, {time.time() - t0:.0f} s", flush=True)
            if out:
                np.savez_compressed(out, **pack())
    data = pack()
    if out:
        np.savez_compressed(out, **data)
    return data


# ---------------------------------------------------------------- network --
class Network:
    """24 -> 64 -> 64 -> K MLP on the GPU (fl_mlp_*), with feature scaling."""

    def __init__(self, n_in=N_FEATURES, h1=64, h2=64, n_out=len(TABLE), seed=1):
        h = C.c_void_p()
        check(load().fl_mlp_create(C.byref(h), n_in, h1, h2, n_out, C.c_ulonglong(seed)))
        self._h = h
        self.shape = (n_in, h1, h2, n_out)
        self.mu = np.zeros(n_in, np.float32)
        self.sd = np.ones(n_in, np.float32)

    @property
    def num_params(self) -> int:
        return int(load().fl_mlp_num_params(self._h))

    def params(self) -> np.ndarray:
        p = np.empty(self.num_params, np.float32)
        check(load().fl_mlp_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32).reshape(-1)
        if p.size != self.num_params:
            raise FastLoadArgumentError(f"set_params: {p.size} values for a network of {self.num_params}")
        check(load().fl_mlp_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    @staticmethod
    def _fp(a):
        return np.ascontiguousarray(a, np.float32).ctypes.data_as(C.POINTER(C.c_float))

    @staticmethod
    def _mat(a, cols: int, what: str, rows: int | None = None) -> np.ndarray:
        """a as a C-contiguous float32 (rows, cols) matrix: the library reads
        rows * cols values from it."""
        a = np.ascontiguousarray(a, np.float32)
        if a.ndim != 2 or a.shape[1] != cols or (rows is not None and a.shape[0] != rows):
            raise FastLoadArgumentError(f"{what}: shape {a.shape}, expected ({'rows' if rows is None else rows}, {cols})")
        return a

    def forward_raw(self, X) -> np.ndarray:
        """Network outputs for already-scaled features."""
        X = self._mat(X, self.shape[0], "forward X")
        Y = np.empty((X.shape[0], self.shape[3]), np.float32)
        check(load().fl_mlp_forward(self._h, self._fp(X), X.shape[0], Y.ctypes.data_as(C.POINTER(C.c_float))))
        return Y

    def grad_raw(self, X, Tg, M=None):
        X = self._mat(X, self.shape[0], "grad X")
        Tg = self._mat(Tg, self.shape[3], "grad targets", X.shape[0])
        Mk = None if M is None else self._mat(M, self.shape[3], "grad mask", X.shape[0])
        loss = np.zeros(1, np.float32)
        g = np.empty(self.num_params, np.float32)
        check(load().fl_mlp_grad(self._h, self._fp(X), self._fp(Tg), None if Mk is None else self._fp(Mk),
                                 X.shape[0], loss.ctypes.data_as(C.POINTER(C.c_float)),
                                 g.ctypes.data_as(C.POINTER(C.c_float))))
        return float(loss[0]), g

    def fit(self, X, times, epochs=3000, lr=3e-3) -> np.ndarray:
        """Trains on features X and measured times (ms per variant, NaN for
        variants the matrix may not use, which the loss masks out)."""
        X = self._mat(X, self.shape[0], "fit X")
        tg, mask = targets(times), mask_of(times)
        Tg = self._mat(tg, self.shape[3], "fit times", X.shape[0])
        M = self._mat(mask, self.shape[3], "fit mask", X.shape[0])
        self.mu = X.mean(0)
        self.sd = X.std(0) + 1e-6
        Xn = np.ascontiguousarray((X - self.mu) / self.sd, np.float32)
        losses = np.empty(epochs, np.float32)
        check(load().fl_mlp_train(self._h, self._fp(Xn), self._fp(Tg), self._fp(M), Xn.shape[0], epochs,
                                  C.c_float(lr), losses.ctypes.data_as(C.POINTER(C.c_float))))
        return losses

    def predict(self, X, allow=None) -> np.ndarray:
        """Variant with the lowest predicted time per row of X, among the
        allowed ones (allow: boolean rows or one row; None = all)."""
        Xn = (np.asarray(X, np.float32) - self.mu) / self.sd
        out = self.forward_raw(Xn).astype(np.float64)
        if allow is not None:
            out = np.where(np.broadcast_to(np.asarray(allow, bool), out.shape), out, np.inf)
        return np.argmin(out, axis=1)

    def close(self):
        if self._h:
            load().fl_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuner_data", "model.fltuner")
_MAGIC = b"FLTUNER1"


def save_model(net: Network, path: str) -> None:
    """The trained network in the library's model format (fl_tune.cu):
    magic, shape, feature scaling, parameters, the variant table."""
    n_in, h1, h2, n_out = net.shape
    opts = np.array([[o[k] for k in _OPT_FIELDS] for o in TABLE], "<i4")
    with open(path, "wb") as f:
        f.write(_MAGIC)
        f.write(np.array([n_in, h1, h2, n_out, len(TABLE), 0, 0, 0], "<i4").tobytes())
        f.write(np.asarray(net.mu, "<f4").tobytes())
        f.write(np.asarray(net.sd, "<f4").tobytes())
        f.write(net.params().astype("<f4").tobytes())
        f.write(opts.tobytes())


def load_model(path: str = MODEL) -> Network:
    """The trained network of `path` on the current device."""
    raw = open(path, "rb").read()
    if raw[:8] != _MAGIC:
        raise ValueError(f"{path}: not a tuner model")
    n_in, h1, h2, n_out, nv = (int(v) for v in np.frombuffer(raw, "<i4", 5, 8))
    if nv != len(TABLE) or n_out != nv:
        raise ValueError(f"{path}: {nv} variants, the library has {len(TABLE)}")
    net = Network(n_in, h1, h2, n_out)
    o = 40
    net.mu = np.frombuffer(raw, "<f4", n_in, o).copy()
    net.sd = np.frombuffer(raw, "<f4", n_in, o + 4 * n_in).copy()
    o += 8 * n_in
    net.set_params(np.frombuffer(raw, "<f4", net.num_params, o))
    o += 4 * net.num_params
    opts = np.frombuffer(raw, "<i4", 8 * nv, o).reshape(nv, 8)
    if any(dict(zip(_OPT_FIELDS, (int(v) for v in row))) != t for row, t in zip(opts, TABLE)):
        raise ValueError(f"{path}: variant table differs from the library's")
    return net


_LOADED: dict = {}


def choose(plan, value_type: int, model: str | None = None) -> tuple[int, str]:
    """(variant index, name) the trained network predicts fastest for this
    plan's matrix among the variants a value_type caller may use -- the
    choice fl_plan_add_tuned_form makes through the C ABI."""
    path = model or MODEL
    net = _LOADED.get(path)
    if net is None:
        net = _LOADED[path] = load_model(path)
    i = int(net.predict(features(plan, value_type)[None, :], allowed(value_type))[0])
    return i, VARIANTS[i]


def mask_of(times) -> np.ndarray:
    return np.isfinite(np.asarray(times, np.float64)).astype(np.float32)


def targets(times) -> np.ndarray:
    """log2(t_variant / t_best) per matrix over the timed variants: 0 for the
    best, 0 (masked) where a variant was not timed."""
    t = np.asarray(times, np.float64)
    best = np.nanmin(t, axis=1, keepdims=True)
    return np.nan_to_num(np.log2(t / best), nan=0.0).astype(np.float32)


def evaluate(pred: np.ndarray, times: np.ndarray) -> dict:
    """Regret of predicted variants against the exhaustive best, and speedup
    over the method without the tuner (the library default) and over the
    plain tile stream."""
    t = np.asarray(times, np.float64)
    idx = np.arange(len(t))
    chosen = t[idx, pred]
    best = np.nanmin(t, axis=1)
    regret = chosen / best - 1.0
    auto = t[:, DEFAULT]
    none = t[:, PLAIN]
    return {
        "matrices": int(len(t)),
        "variants": int(t.shape[1]),
        "mean_regret": float(regret.mean()),
        "median_regret": float(np.median(regret)),
        "frac_within_10pct": float((regret <= 0.10).mean()),
        "total_time_regret": float(chosen.sum() / best.sum() - 1.0),
        "speedup_vs_auto_rule": float(auto.sum() / chosen.sum()),
        "speedup_vs_plain_tiles": float(none.sum() / chosen.sum()),
        "auto_rule_mean_regret": float((auto / best - 1.0).mean()),
        "geomean_speedup_vs_auto_rule": float(np.exp(np.mean(np.log(auto / chosen)))),
    }


def train_and_evaluate(data: dict, n_train: int = 2000, epochs: int = 3000, seed: int = 1, save: str | None = None):
    X, T = np.asarray(data["X"]), np.asarray(data["T"])
    net = Network(seed=seed)
    losses = net.fit(X[:n_train], T[:n_train], epochs=epochs)
    allow = np.isfinite(T)
    res = {"train": evaluate(net.predict(X[:n_train], allow[:n_train]), T[:n_train]),
           "heldout": (evaluate(net.predict(X[n_train:], allow[n_train:]), T[n_train:])
                       if len(X) > n_train else None),
           "final_loss": float(losses[-1]) if len(losses) else None, "epochs": epochs}
    if save:
        save_model(net, save)
        res["model"] = save
    net.close()
    return res


def main():
    ap = argparse.ArgumentParser(prog="python -m fastload_gb300.tuner")
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--count", type=int, default=2200)
    c.add_argument("--seed", type=int, default=5)
    c.add_argument("--out", required=True)
    t = sub.add_parser("train", help="train on the first --train matrices and save the model")
    t.add_argument("--data", required=True)
    t.add_argument("--train", type=int, default=2000)
    t.add_argument("--epochs", type=int, default=3000)
    t.add_argument("--seed", type=int, default=1)
    t.add_argument("--out", default=MODEL)
    e = sub.add_parser("evaluate")
    e.add_argument("--data", required=True)
    e.add_argument("--train", type=int, default=2000)
    e.add_argument("--epochs", type=int, default=3000)
    a = ap.parse_args()
    if a.cmd == "collect":
        collect(a.count, a.seed, a.out)
        return
    with np.load(a.data) as z:
        data = {k: z[k] for k in z.files}
    if a.cmd == "train":
        print(json.dumps(train_and_evaluate(data, a.train, a.epochs, a.seed, save=a.out)))
    else:
        print(json.dumps(train_and_evaluate(data, a.train, a.epochs)))


if __name__ == "__main__":
    main()
