"""Learned tuner: picks the heavy band (bucket threshold) / kernel variant of a
matrix from 24 features with a small MLP trained on the project's own
exhaustive autotuner timings.

Variants (one class each):
    none   FastLoad tile stream only (no heavy band; one atomic per run)
    2048   densest 2048 sorted columns as row slices, x in shared memory
    8192   densest 8192 columns
    max    the widest band whose x fits shared memory (24576 FP64 / 49152 FP32)
    all    every column as row slices (rows owned by one lane, no atomics)
    auto   the library's static rule (plan default) -- the method without the tuner

The training set: seeded matrices of five families (uniform rows, Zipf
column degrees, banded, block-diagonal, row-skewed) generated on the GPU
(fl_gen_fill), n log-uniform in [1e4, 4e6], nnz log-uniform in [1e5, 6e7],
FP64 or FP32 values.  The network (24 -> 64 -> 64 -> 6, ReLU) regresses
log2(t_variant / t_best) and is trained on the GPU by the library's own
forward/backward/Adam kernels (fl_mlp_*); the autotuner's measurements are
what regret is measured against.

    python -m fastload_gb300.tuner collect --count 2200 --out data.npz
    python -m fastload_gb300.tuner evaluate --data data.npz
"""
from __future__ import annotations

import argparse
import os
import ctypes as C
import json
import time

import numpy as np

from ._lib import FastLoadArgumentError, check, load

FAMILIES = ("uniform", "zipf", "banded", "blockdiag", "rowskew")
VARIANTS = ("none", "2048", "8192", "max", "all", "auto")
N_FEATURES = 24
N_RANGE = (1e4, 4e6)
NNZ_RANGE = (1e5, 6e7)


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


def make_plan(spec: dict, heavy_band: int = -1):
    """Generates the spec's matrix on the GPU and builds its plan.
    Returns (plan, nnz, device x)."""
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
    plan = Plan.from_csc(spec["m"], spec["n"], cp, rows[:nnz], vals[:nnz], heavy_band=heavy_band)
    g = torch.Generator(device="cuda")
    g.manual_seed(spec["seed"] & 0x7FFFFFFF)
    x = torch.rand(spec["n"], dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    del rows, vals, cp
    return plan, nnz, x


def features(plan, value_type: int) -> np.ndarray:
    out = np.zeros(N_FEATURES, np.float32)
    check(load().fl_plan_features(plan._h, int(value_type), out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


# ------------------------------------------------------------- autotune --
def variant_band(variant: str, value_type: int) -> int:
    from .plan import BAND_ALL, BAND_AUTO, BAND_NONE

    return {"none": BAND_NONE, "2048": 2048, "8192": 8192, "max": 24576 if value_type == 0 else 49152,
            "all": BAND_ALL, "auto": BAND_AUTO}[variant]


def autotune(plan, x, value_type: int, reps: int = 5) -> np.ndarray:
    """Exhaustive: builds every variant as a form of the plan and times one
    SpMV (median of reps, L2 flushed before each).  Returns ms per variant."""
    import torch

    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    xs = plan.permute_x_k(x, k=1, to_f32=value_type != 0)
    y = torch.empty(plan.m, dtype=torch.float64, device="cuda")
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = np.zeros(len(VARIANTS))
    for vi, v in enumerate(VARIANTS):
        band = variant_band(v, value_type)
        if isinstance(band, int) and band > plan.n:
            band = -2  # wider than the matrix: every column
        fid = plan.add_form(value_type, band)
        plan.spmv_form(fid, xs, y)
        ts = []
        for _ in range(reps):
            flush.zero_()
            a.record()
            plan.spmv_form(fid, xs, y)
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        times[vi] = float(np.median(ts))
    plan.check()
    return times


def collect(count: int, seed: int = 5, out: str | None = None, log_every: int = 50) -> dict:
    rng = np.random.default_rng(seed)
    X, T, meta = [], [], []
    t0 = time.time()
    def pack():
        return {"X": np.array(X, np.float32).reshape(-1, N_FEATURES), "T": np.array(T, np.float64),
                "meta": np.array([json.dumps(m) for m in meta]), "variants": np.array(VARIANTS)}

    for i in range(count):
        spec = sample_spec(rng, i)
        plan, nnz, x = make_plan(spec)
        try:
            f = features(plan, spec["values"])
            t = autotune(plan, x, spec["values"])
        finally:
            plan.close()
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

    def __init__(self, n_in=N_FEATURES, h1=64, h2=64, n_out=len(VARIANTS), seed=1):
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
        """Trains on features X and measured times (ms per variant)."""
        X = self._mat(X, self.shape[0], "fit X")
        Tg = self._mat(targets(times), self.shape[3], "fit times", X.shape[0])
        self.mu = X.mean(0)
        self.sd = X.std(0) + 1e-6
        Xn = np.ascontiguousarray((X - self.mu) / self.sd, np.float32)
        losses = np.empty(epochs, np.float32)
        check(load().fl_mlp_train(self._h, self._fp(Xn), self._fp(Tg), None, Xn.shape[0], epochs, C.c_float(lr),
                                  losses.ctypes.data_as(C.POINTER(C.c_float))))
        return losses

    def predict(self, X) -> np.ndarray:
        Xn = (np.asarray(X, np.float32) - self.mu) / self.sd
        return np.argmin(self.forward_raw(Xn), axis=1)

    def close(self):
        if self._h:
            load().fl_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuner_data", "model.npz")


def save_model(net: Network, path: str) -> None:
    """Weights, feature scaling, shape and variant names of a trained network."""
    np.savez_compressed(path, params=net.params(), mu=net.mu, sd=net.sd, shape=np.array(net.shape),
                        variants=np.array(VARIANTS))


def load_model(path: str = MODEL) -> Network:
    """The trained network of `path` on the current device."""
    with np.load(path) as z:
        shape = tuple(int(v) for v in z["shape"])
        if tuple(str(v) for v in z["variants"]) != VARIANTS:
            raise ValueError(f"{path}: variants {list(z['variants'])} differ from {list(VARIANTS)}")
        net = Network(*shape)
        net.set_params(z["params"])
        net.mu = z["mu"].astype(np.float32)
        net.sd = z["sd"].astype(np.float32)
    return net


_LOADED: dict = {}


def choose(plan, value_type: int, model: str | None = None) -> tuple[str, int]:
    """(variant, heavy band) the trained network predicts fastest for this
    plan's matrix in the given value type."""
    path = model or MODEL
    net = _LOADED.get(path)
    if net is None:
        net = _LOADED[path] = load_model(path)
    v = VARIANTS[int(net.predict(features(plan, value_type)[None, :])[0])]
    band = variant_band(v, value_type)
    if band > plan.n:
        band = variant_band("all", value_type)
    return v, band


def targets(times) -> np.ndarray:
    """log2(t_variant / t_best) per matrix: 0 for the best variant."""
    t = np.asarray(times, np.float64)
    return np.log2(t / t.min(axis=1, keepdims=True)).astype(np.float32)


def evaluate(pred: np.ndarray, times: np.ndarray) -> dict:
    """Regret of predicted variants against the exhaustive best, and speedup
    over the method without the tuner (the 'auto' rule) and over the plain
    tile stream ('none')."""
    t = np.asarray(times, np.float64)
    idx = np.arange(len(t))
    chosen = t[idx, pred]
    best = t.min(axis=1)
    regret = chosen / best - 1.0
    auto = t[:, VARIANTS.index("auto")]
    none = t[:, VARIANTS.index("none")]
    return {
        "matrices": int(len(t)),
        "mean_regret": float(regret.mean()),
        "median_regret": float(np.median(regret)),
        "frac_within_10pct": float((regret <= 0.10).mean()),
        "total_time_regret": float(chosen.sum() / best.sum() - 1.0),
        "speedup_vs_auto_rule": float(auto.sum() / chosen.sum()),
        "speedup_vs_plain_tiles": float(none.sum() / chosen.sum()),
        "auto_rule_mean_regret": float((auto / best - 1.0).mean()),
        "geomean_speedup_vs_auto_rule": float(np.exp(np.mean(np.log(auto / chosen)))),
    }


def train_and_evaluate(data: dict, n_train: int = 2000, epochs: int = 3000, seed: int = 1) -> dict:
    X, T = np.asarray(data["X"]), np.asarray(data["T"])
    net = Network(seed=seed)
    losses = net.fit(X[:n_train], T[:n_train], epochs=epochs)
    res = {"train": evaluate(net.predict(X[:n_train]), T[:n_train]),
           "heldout": evaluate(net.predict(X[n_train:]), T[n_train:]) if len(X) > n_train else None,
           "final_loss": float(losses[-1]) if len(losses) else None, "epochs": epochs}
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
        X, T = np.asarray(data["X"]), np.asarray(data["T"])
        net = Network(seed=a.seed)
        losses = net.fit(X[:a.train], T[:a.train], epochs=a.epochs)
        save_model(net, a.out)
        res = {"train": evaluate(net.predict(X[:a.train]), T[:a.train]),
               "heldout": evaluate(net.predict(X[a.train:]), T[a.train:]) if len(X) > a.train else None,
               "final_loss": float(losses[-1]), "model": a.out}
        net.close()
        print(json.dumps(res))
    else:
        print(json.dumps(train_and_evaluate(data, a.train, a.epochs)))


if __name__ == "__main__":
    main()
