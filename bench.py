"""FastLoad SpMV benchmark (one JSON line on rank 0).

Workload: the plain FP64 FastLoad SpMV at scale -- square n = 1,048,576,
column degrees Zipf(1.8) capped at 50,000 (about 20-27M nonzeros, seed 2),
distinct uniform rows, values N(0,1), x U[-1,1].  A step is one y = A x over
the whole matrix (y zeroed, then the FastLoad kernel) with the layout and
sorted x resident in HBM.

metric/unit: achieved SpMV bandwidth in GB/s by the algorithmic byte count
B = nnz*(8+4) + (n+1)*4 + n*8 + m*8 (FP64 values, int32 rows, FP64 x and y),
with GFLOP/s (2 nnz per SpMV), % of the measured HBM peak and the relative
error against the compensated CPU FP64 oracle reported beside it.

--impl reference times the reference's CPU implementation of the path (the
oracle's port of FastLoad_cpu, src/FastLoad_CPU.h:19-31, spread over all host
threads with atomic y updates as in test.cu:46-57) on bounded samples of the
same workload.  Under torchrun (N > 1) every rank runs an independent
replica (the path has no exchange step); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpMV HBM GB/s (% of peak) and GFLOP/s vs plain FP64 kernel at stated error"
SEED = 2
N_COLS = 1 << 20
WORKLOAD = "fastload_fp64_zipf1.8_n1048576_cap50000"
DATA = ("synthetic: seeded Zipf(1.8) column degrees capped at 50,000, distinct uniform rows, N(0,1) values, "
        "U[-1,1] x (stands in for the SuiteSparse matrices the reference is run on)")


def algorithmic_bytes(m, n, nnz, s_val=8, s_idx=4, s_x=8, s_y=8, k=1):
    return nnz * (s_val + s_idx) + (n + 1) * 4 + k * n * s_x + k * m * s_y


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def world_max(x: float, dist, device: str) -> float:
    """Max of x over the ranks (the slowest replica sets the job's time);
    x itself without a process group.  device: "cuda" for NCCL, "cpu" for gloo."""
    if not dist:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(bytes_per_step: float, world: int, ms_per_step: float) -> float:
    """Whole-job GB/s of `world` independent replicas, each moving
    bytes_per_step per step, timed by the slowest rank."""
    return bytes_per_step * world / (ms_per_step * 1e-3) / 1e9


def ncu_traffic(kernel, workload):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary
    (profiles/ncu_traffic.txt: '<kernel> <workload> <bytes>' lines)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        f = ln.split()
        if len(f) >= 3 and f[0] == kernel and f[1] == workload:
            return float(f[2])
    return None


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        # the raw samples; FL_CLOCKS_DIR keeps them somewhere that outlives the run
        out_dir = os.environ.get("FL_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self, t0, t1):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for ln in open(self.path):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        busy = [s for s, _, _ in rows]
        return {"sm_mhz": float(np.median(busy)), "sm_max_mhz": max(x for _, x, _ in rows), "reasons": reasons,
                "samples": len(rows)}


def _gen():
    """fastload_gb300/gen.py (numpy only), loaded by path: importing the
    package would load the CUDA library, which the CPU reference arm must
    not map."""
    import importlib.util

    mod = sys.modules.get("fastload_gb300.gen")
    if mod is not None:
        return mod
    spec = importlib.util.spec_from_file_location("fastload_gb300_gen", os.path.join(ROOT, "fastload_gb300", "gen.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod  # dataclasses look their module up while the class is made
    spec.loader.exec_module(mod)
    return mod


def make_workload(n=N_COLS):
    return _gen().zipf_columns(n, 1.8, 50000, seed=SEED)


def bench_config(c, world):
    """The workload description both arms print (identical dicts)."""
    return {"workload": workload_name(c.n), "m": c.m, "n": c.n, "nnz": c.nnz, "seed": SEED,
            "values": "f64", "l2": "inputs larger than L2: matrix streams %.0f MB vs 129 MB L2" % (c.nnz * 12 / 1e6),
            "parallelism": f"replicas x{world}"}


def workload_name(n):
    return WORKLOAD if n == N_COLS else f"fastload_fp64_zipf1.8_n{n}_cap50000"


def cpu_baseline_sample(c, budget_s=12.0, threads=1):
    """Times the oracle's FastLoad_cpu port over whole passes of the matrix
    for about budget_s seconds; returns GB/s by the same byte count."""
    import oracle

    lay = oracle.build(c.m, c.n, csc=(c.colptr, c.rowidx, c.val), x=c.x)
    B = algorithmic_bytes(c.m, c.n, c.nnz)
    passes, t = 0, 0.0
    used = 1
    while t < budget_s or passes == 0:
        t0 = time.perf_counter()
        if threads == 1:
            oracle.fastload_spmv(lay, lay["sortx"], c.m)
        else:
            _, used = oracle.fastload_spmv(lay, lay["sortx"], c.m, threads=threads)
        t += time.perf_counter() - t0
        passes += 1
        if passes >= 200:
            break
    return {"value": B * passes / t / 1e9, "unit": "GB/s", "cores": used, "kind": "port",
            "sample": f"{passes} full passes of the FastLoad_cpu tile loop (src/FastLoad_CPU.h:19-31) over the "
                      f"same matrix ({c.nnz} nonzeros), {t:.1f} s"}


def run_reference(args, rank, world):
    """--impl reference: the CPU implementation on all host threads."""
    if rank != 0:
        return
    import oracle

    c = make_workload(args.cols)
    lay = oracle.build(c.m, c.n, csc=(c.colptr, c.rowidx, c.val), x=c.x)
    T = int(lay["tilenum"])
    # each step: a bounded, rotating sample of about 1/16 of the tiles
    nsamp = 16
    cuts = np.searchsorted(lay["tile_ptr"], np.linspace(0, c.nnz, nsamp + 1).astype(np.int64))
    cuts[0], cuts[-1] = 0, T
    threads = os.cpu_count() or 1

    def step(i):
        a, b = int(cuts[i % nsamp]), int(cuts[i % nsamp + 1])
        sub = {"tilenum": b - a, "tile_ptr": lay["tile_ptr"][a:b + 1] - 0, "tile_len": lay["tile_len"][a:b],
               "tile_colidx": lay["tile_colidx"][a:b], "sortrowidx": lay["sortrowidx"], "sortval": lay["sortval"]}
        y, used = oracle.fastload_spmv(sub, lay["sortx"], c.m, threads=threads)
        return int(lay["tile_ptr"][b] - lay["tile_ptr"][a]), used

    for i in range(args.warmup):
        step(i)
    nz_total, used = 0, 1
    t0 = time.perf_counter()
    for i in range(args.steps):
        nz, used = step(i)
        nz_total += nz
    t = time.perf_counter() - t0
    frac = nz_total / c.nnz
    B = algorithmic_bytes(c.m, c.n, c.nnz) * frac
    gbs = B / t / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": bench_config(c, world),
            "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": used, "kind": "port",
                             "sample": f"{args.steps} steps, each 1/{nsamp} of the tiles in turn, FastLoad_cpu "
                                       f"tile loop on {used} OpenMP threads with atomic y updates"},
            "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _time_ms(fn, reps, flush=None):
    """Mean device time of fn() over reps, with an optional L2 flush before
    each timed call (events bracket fn only)."""
    import torch

    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        fn()
    ts = []
    for _ in range(reps):
        if flush is not None:
            flush.zero_()
        a.record()
        fn()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.mean(ts))


def _time_b2b_ms(fns, launches=60):
    """Mean device time of one call over `launches` calls made back to back
    between two events, cycling through fns (one callable per copy of the
    data, so each call's streams were evicted from L2 by the other copies'
    calls), after a device sleep that lets the host enqueue ahead."""
    import torch

    for f in fns * 3:
        f()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda._sleep(2_000_000)
    a.record()
    for i in range(launches):
        fns[i % len(fns)]()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / launches


def measure_forms(fl, peak, reps=20):
    """Storage / multi-RHS forms against the plain FP64 kernel on the same
    inputs: the 128^3 7-point Laplacian (k = 1 and 8) and the Zipf matrix.
    GB/s by each form's algorithmic bytes.  `ms` is the steady state of the
    bench step: calls back to back alternating between two copies of the
    matrix's plan (the two copies' streams exceed the 129 MB L2, so no call
    finds its matrix in L2; x stays there, as in an iterative solver);
    `ms_cold` is one call after a 256 MB write that flushes L2 (x, y and
    the streams cold, launch and start-up unhidden)."""
    import torch

    import oracle
    from fastload_gb300 import gen

    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    out = {}

    def entry(c, t_ms, t_cold, k, s_val, s_x, y, yref, plain_gflops=None):
        B = algorithmic_bytes(c.m, c.n, c.nnz, s_val=s_val, s_idx=4, s_x=s_x, s_y=8, k=k)
        gflops = 2.0 * c.nnz * k / (t_ms * 1e-3) / 1e9
        nw, mx = oracle.rel_errors(np.asarray(y).reshape(-1), np.asarray(yref).reshape(-1))
        d = {"ms": t_ms, "gbs": B / (t_ms * 1e-3) / 1e9, "pct_of_peak": 100.0 * B / (t_ms * 1e-3) / 1e9 / peak,
             "gflops": gflops, "ms_cold": t_cold, "pct_of_peak_cold": 100.0 * B / (t_cold * 1e-3) / 1e9 / peak,
             "rel_err_normwise": nw, "rel_err_max": mx, "bytes": B}
        if plain_gflops:
            d["gflops_vs_plain_fp64"] = gflops / plain_gflops
        return d

    forms = [("f64", fl.VALUES_F64, 8), ("f32", fl.VALUES_F32, 4), ("bf16x2", fl.VALUES_BF16X2, 4)]
    cases = [("lap128", gen.laplacian7(128, seed=4), [("band_none", fl.BAND_NONE), ("band_all", fl.BAND_ALL)]),
             ("zipf_n1048576", make_workload(N_COLS), [("band_auto", fl.BAND_AUTO), ("band_none", fl.BAND_NONE)])]
    for cname, c, bands in cases:
        rng = np.random.default_rng(11)
        x8 = rng.uniform(-1, 1, c.n * 8)
        ref = {1: oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x)}
        if not cname.startswith("zipf"):
            ref[8] = oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, x8, k=8)
        xin = {1: c.x, 8: x8}
        plans = [fl.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) for _ in range(2)]
        p = plans[0]
        xs = p.permute_x(torch.from_numpy(c.x).cuda())
        y = torch.empty(c.m, dtype=torch.float64, device="cuda")

        def both(call):
            return [lambda q=q: call(q) for q in plans]

        # the plain FP64 kernel the forms are compared with: the plan's
        # default (FL_KERNEL_AUTO), the drop-in FastLoad_spmv path
        t = _time_b2b_ms(both(lambda q: q.spmv(xs, y, kernel=fl.KERNEL_AUTO)))
        tc = _time_ms(lambda: p.spmv(xs, y, kernel=fl.KERNEL_AUTO), reps, flush)
        plain = entry(c, t, tc, 1, 8, 8, y.cpu().numpy(), ref[1])
        out[f"{cname}_plain_fp64_auto_k1"] = plain
        # context: the pure FastLoad tile stream (one atomic per run)
        t = _time_b2b_ms(both(lambda q: q.spmv(xs, y, kernel=fl.KERNEL_STREAM2)))
        tc = _time_ms(lambda: p.spmv(xs, y, kernel=fl.KERNEL_STREAM2), reps, flush)
        out[f"{cname}_fp64_stream_k1"] = entry(c, t, tc, 1, 8, 8, y.cpu().numpy(), ref[1], plain["gflops"])
        for bname, band in bands:
            for fname, vt, sv in forms:
                fids = [q.add_form(vt, band) for q in plans]
                for k in (1, 8):
                    if cname.startswith("zipf") and k == 8:
                        continue
                    xk = p.permute_x_k(torch.from_numpy(xin[k]).cuda(), k=k, to_f32=vt != fl.VALUES_F64)
                    yk = torch.empty(c.m * k, dtype=torch.float64, device="cuda")
                    calls = [lambda q=q, f=f: q.spmv_form(f, xk, yk, k=k) for q, f in zip(plans, fids)]
                    t = _time_b2b_ms(calls)
                    tc = _time_ms(calls[0], reps, flush)
                    sx = 8 if vt == fl.VALUES_F64 else 4
                    out[f"{cname}_{fname}_{bname}_k{k}"] = entry(
                        c, t, tc, k, sv, sx, yk.cpu().numpy(), ref[k], plain["gflops"])
        # the learned tuner's pick for this matrix (through the C ABI), for
        # FP64 and FP32 callers (an FP32 caller may get BF16 hi+lo storage)
        for fname, vt, sv in forms[:2]:
            picks = [q.add_tuned_form(vt) for q in plans]
            fids = [f for f, _ in picks]
            info = p.form_info(fids[0])
            xk = p.permute_x_k(torch.from_numpy(xin[1]).cuda(), k=1, to_f32=info["value_type"] != fl.VALUES_F64)
            yk = torch.empty(c.m, dtype=torch.float64, device="cuda")
            calls = [lambda q=q, f=f: q.spmv_form(f, xk, yk) for q, f in zip(plans, fids)]
            t = _time_b2b_ms(calls)
            tc = _time_ms(calls[0], reps, flush)
            d = entry(c, t, tc, 1, sv, 8 if vt == fl.VALUES_F64 else 4, yk.cpu().numpy(), ref[1], plain["gflops"])
            d["tuned_variant"] = picks[0][1]
            out[f"{cname}_{fname}_tuned_k1"] = d
        for q in plans:
            q.check()
            q.close()
        del c
    return out


def measure_batch(fl, peak, reps=10):
    """Batched form: 256 independent seeded matrices (n log-uniform in
    [1e3, 2e5], mean degree U[4, 32], half Poisson and half Zipf(1.5) column
    degrees), FP32 values with FP32 accumulation, one persistent launch,
    direct and replayed from a captured CUDA graph; against the plain FP64
    kernel (each plan's default, FL_KERNEL_AUTO) launched once per matrix on
    the same inputs.  Calls back to back (the slices exceed L2), plus one
    cold call after an L2 flush (`ms_cold`)."""
    import torch

    import oracle
    from fastload_gb300 import gen

    mats = gen.batch(256, seed=3, dtype=np.float64)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    plans = [fl.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) for c in mats]
    prep = time.perf_counter() - t0
    nnz = sum(c.nnz for c in mats)
    M, N = sum(c.m for c in mats), sum(c.n for c in mats)
    x = torch.from_numpy(np.concatenate([c.x for c in mats])).cuda()
    out = {"matrices": len(mats), "nnz": nnz, "rows": M, "plan_build_s": prep}
    # plain FP64 kernel, one launch per matrix
    xs64 = [p.permute_x(torch.from_numpy(c.x).cuda()) for p, c in zip(plans, mats)]
    ys64 = [torch.empty(c.m, dtype=torch.float64, device="cuda") for c in mats]

    def plain():
        for p, xs_, y_ in zip(plans, xs64, ys64):
            p.spmv(xs_, y_, kernel=fl.KERNEL_AUTO)

    t_plain = _time_b2b_ms([plain], 10)
    out["plain_fp64_per_matrix"] = {"ms": t_plain, "gflops": 2.0 * nnz / (t_plain * 1e-3) / 1e9, "launches": len(mats)}
    with fl.Batch(plans, value_type=fl.VALUES_F32, y_f32=True) as b:
        for p in plans:
            p.close()
        xs = b.permute_x(x)
        y = torch.empty(b.m, dtype=torch.float32, device="cuda")
        # the batch's slices (1.5 GB) exceed L2: calls back to back
        t_direct = _time_b2b_ms([lambda: b.spmv(xs, y)], 20)
        t_graph = _time_b2b_ms([lambda: b.spmv_graph(xs, y)], 20)
        t_cold = _time_ms(lambda: b.spmv_graph(xs, y), reps, flush)
        yh = y.double().cpu().numpy()
    errs = [oracle.rel_errors(yh[b.m_off[i]:b.m_off[i + 1]],
                              oracle.csc_spmv_dd(c.m, c.n, c.colptr, c.rowidx, c.val, c.x))[0]
            for i, c in enumerate(mats)]
    worst = float(np.max(errs))  # NaN if any matrix's error is
    Bf = nnz * 8 + (N + len(mats)) * 4 + N * 4 + M * 4
    for name, t in (("batch_fp32_direct", t_direct), ("batch_fp32_graph", t_graph)):
        out[name] = {"ms": t, "gbs": Bf / (t * 1e-3) / 1e9, "pct_of_peak": 100.0 * Bf / (t * 1e-3) / 1e9 / peak,
                     "gflops": 2.0 * nnz / (t * 1e-3) / 1e9, "launches": 1,
                     "gflops_vs_plain_fp64": t_plain / t, "rel_err_normwise_worst_matrix": worst,
                     "ms_cold": t_cold, "pct_of_peak_cold": 100.0 * Bf / (t_cold * 1e-3) / 1e9 / peak}
    return out


def measure_comparators(fl, c, x, ydd, B, reps=20):
    """The reference's comparators on the bench matrix, timed like the
    FastLoad kernel (CUDA events per launch, y zeroing outside): its naive
    CSC kernel and cuSPARSE CSR SpMV (each algorithm, handle prepared once).
    GB/s use the same algorithmic bytes as the FastLoad line."""
    import scipy.sparse as sp
    import torch

    import oracle
    from fastload_gb300 import compare

    stream = torch.cuda.current_stream()
    dev = lambda a, t: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", t)  # noqa: E731
    cp, cr, cv = dev(c.colptr, torch.int32), dev(c.rowidx, torch.int32), dev(c.val, torch.float64)
    y = torch.zeros(c.m, dtype=torch.float64, device="cuda")
    out = {}

    def timed(fn, n_reps):
        for _ in range(3):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ts = []
        for _ in range(n_reps):
            y.zero_()
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.mean(ts))

    def entry(ms):
        err = oracle.rel_errors(y.cpu().numpy(), ydd)
        return {"ms": ms, "gbs": B / (ms * 1e-3) / 1e9, "gflops": 2.0 * c.nnz / (ms * 1e-3) / 1e9,
                "rel_err_normwise": err[0]}

    ms = timed(lambda: compare.csc_spmv_naive(c.m, cp, cr, cv, x, y=y, accumulate=True), reps)
    out["naive_csc"] = entry(ms)
    del cp, cr, cv
    A = sp.csc_matrix((c.val, c.rowidx, c.colptr), shape=(c.m, c.n)).tocsr()
    rp, ci, v = dev(A.indptr, torch.int32), dev(A.indices, torch.int32), dev(A.data, torch.float64)
    for alg, name in ((0, "cusparse_csr_default"), (1, "cusparse_csr_alg1"), (2, "cusparse_csr_alg2")):
        try:
            with compare.CuSparse(c.m, c.n, rp, ci, v, alg=alg) as cs:
                out[name] = entry(timed(lambda: cs.spmv(x, y=y), reps))
        except fl.FastLoadError as e:
            out[name] = {"unavailable": str(e)}
    return out


def run_profile(spec):
    """--profile case:values:band:k -- builds one case and runs one kernel a
    few times (for ncu captures).  case lap128 | zipf | zipf<n> | batch (the
    256-matrix batch of the batch line, FP32 values and y; values and band
    are ignored); values f64 | f32 | bf16x2 | plain (the plain FP64 stream
    kernel) | bucket (the FP64 bucketed kernel); band auto | none | all |
    <columns>; k 1 | 8."""
    import torch

    import fastload_gb300 as fl
    from fastload_gb300 import gen

    case, vals, band, k = spec.split(":")
    k = int(k)
    if case == "batch":
        mats = gen.batch(256, seed=3, dtype=np.float64)
        plans = [fl.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) for c in mats]
        with fl.Batch(plans, value_type=fl.VALUES_F32, y_f32=True) as b:
            for p in plans:
                p.close()
            xs = b.permute_x(torch.from_numpy(np.concatenate([c.x for c in mats])).cuda())
            y = torch.empty(b.m, dtype=torch.float32, device="cuda")
            ms = _time_ms(lambda: b.spmv(xs, y), 5)
        print(json.dumps({"profile": spec, "nnz": int(sum(c.nnz for c in mats)), "ms": ms}), flush=True)
        return
    if case == "lap128":
        c = gen.laplacian7(128, seed=4)
    else:
        c = make_workload(int(case[4:]) if case != "zipf" else N_COLS)
    with fl.Plan.from_csc(c.m, c.n, c.colptr, c.rowidx, c.val) as p:
        x = torch.from_numpy(np.random.default_rng(11).uniform(-1, 1, c.n * k)).cuda()
        if vals in ("plain", "bucket"):
            xs = p.permute_x(x[: c.n])
            y = torch.empty(c.m, dtype=torch.float64, device="cuda")
            kern = fl.KERNEL_STREAM2 if vals == "plain" else fl.KERNEL_BUCKET
            fn = lambda: p.spmv(xs, y, kernel=kern)  # noqa: E731
        else:
            vt = {"f64": fl.VALUES_F64, "f32": fl.VALUES_F32, "bf16x2": fl.VALUES_BF16X2}[vals]
            bd = {"auto": fl.BAND_AUTO, "none": fl.BAND_NONE, "all": fl.BAND_ALL}.get(band)
            fid = p.add_form(vt, bd if bd is not None else int(band))
            xs = p.permute_x_k(x, k=k, to_f32=vt != fl.VALUES_F64)
            y = torch.empty(c.m * k, dtype=torch.float64, device="cuda")
            fn = lambda: p.spmv_form(fid, xs, y, k=k)  # noqa: E731
        ms = _time_ms(fn, 5)
        p.check()
    print(json.dumps({"profile": spec, "nnz": c.nnz, "ms": ms}), flush=True)


def run_gpu(args, rank, world):
    import torch

    import fastload_gb300 as fl
    import oracle

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    c = make_workload(args.cols)
    m, n, nnz = c.m, c.n, c.nnz
    B = algorithmic_bytes(m, n, nnz)
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    plan = fl.Plan.from_csc(m, n, c.colptr, c.rowidx, c.val, with_reference_arrays=True)
    torch.cuda.synchronize()
    prep_s = time.perf_counter() - t0
    x = torch.from_numpy(c.x).cuda()
    xs = plan.permute_x(x)
    y = torch.zeros(m, dtype=torch.float64, device="cuda")
    kernel = fl.KERNEL_AUTO

    # error statement against the compensated FP64 oracle
    ydd = oracle.csc_spmv_dd(m, n, c.colptr, c.rowidx, c.val, c.x)
    plan.spmv(xs, y)
    rel = oracle.rel_errors(y.cpu().numpy(), ydd)

    # One step is y = A xs: the library's y-zeroing kernel and the SpMV
    # kernel, the second launched as a programmatic dependent of the first
    # (and the next step's zeroing of this step's SpMV), so launches overlap
    # their start-up.  Events only at the ends of the region: an event
    # recorded between two launches serialises them.
    def step():
        plan.spmv(xs, y, kernel=kernel)

    launches_per_step = plan.info["spmv_launches"]
    K = args.steps
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kstart, kend = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        # warm-up inside the sampled region, right before the timed steps
        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        # A device sleep (about a millisecond) ahead of the start event lets
        # the host enqueue the first steps before the event fires, so the
        # K steps run back to back on the device from the start event on and
        # a short run (K = 20) does not carry the host's first-launch latency.
        torch.cuda._sleep(2_000_000)
        wall0 = time.time()
        start.record(stream)
        for i in range(K):
            step()
        end.record(stream)
        torch.cuda.synchronize()
        wall1 = time.time()
        # the SpMV kernel alone, K launches back to back accumulating into y:
        # its average duration for the roofline
        kstart.record(stream)
        for i in range(K):
            plan.spmv(xs, y, accumulate=True, kernel=kernel)
        kend.record(stream)
        torch.cuda.synchronize()
        wall2 = time.time()
    if dist:
        dist.barrier()
    total_ms = start.elapsed_time(end)
    kern_ms = kstart.elapsed_time(kend) / K
    total_ms = world_max(total_ms, dist, "cuda")
    ms_step = total_ms / K
    peak, peak_kind = measured_peaks()
    value = replica_value(B, world, ms_step)
    achieved = B / (kern_ms * 1e-3) / 1e9

    # one launch at a time (the reference-design kernel, the other variants):
    # a ~50 us device sleep ahead of the start event lets the host enqueue the
    # launch first, so the events bracket device time, not host launch latency
    def time_kernel(kern, reps=50):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(3):
            plan.spmv(xs, y, kernel=kern)
        ts = []
        for _ in range(reps):
            y.zero_()
            torch.cuda._sleep(100_000)
            a.record(stream)
            plan.spmv(xs, y, accumulate=True, kernel=kern)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.mean(ts))

    kernels = [("tile", fl.KERNEL_TILE), ("stream1", fl.KERNEL_STREAM), ("stream2", fl.KERNEL_STREAM2)]
    if plan.info["heavy_cols"]:
        kernels.append(("bucket", fl.KERNEL_BUCKET))
    variants = {} if args.quick else {name: B / (time_kernel(k) * 1e-3) / 1e9 for name, k in kernels}
    kern_iso_ms = time_kernel(kernel, reps=10 if args.quick else 50)

    # end to end through the host-buffer C-ABI: each step uploads x from
    # pinned host memory, computes y = A x and downloads y.  The pipelined
    # call lets consecutive steps overlap (upload of one x and download of an
    # earlier y while a kernel computes); the synchronous call is one step's
    # latency.
    xs_host = plan.permute_x(x).cpu()
    hx_t = [xs_host.clone().pin_memory() for _ in range(2)]
    hy_t = [torch.empty(m, dtype=torch.float64).pin_memory() for _ in range(2)]
    hx, hy = [t.numpy() for t in hx_t], [t.numpy() for t in hy_t]
    # steady-state throughput of the pipelined call: at least 100 calls, so
    # the pipeline's fill (first upload) and drain (last download) are a
    # small part of the measured span whatever K is
    ke = 3 if args.quick else max(100, min(K, 400))
    for i in range(4):
        plan.spmv_host_async(hx[i % 2], hy[i % 2], kernel=kernel)
    stream.synchronize()
    t0 = time.perf_counter()
    for i in range(ke):
        plan.spmv_host_async(hx[i % 2], hy[i % 2], kernel=kernel)
    stream.synchronize()
    e2e_s = (time.perf_counter() - t0) / ke
    e2e_rel = float(np.max([oracle.rel_errors(hy[0], ydd)[0], oracle.rel_errors(hy[1], ydd)[0]]))
    # the synchronous call overlaps its own upload with the kernel, whose
    # light items wait (bounded) for a flag written on a second stream; a
    # profiler that serialises the GPU's work would let that wait expire, so
    # --quick (the profiling mode) leaves it out
    sync_call = None
    if not args.quick:
        for _ in range(3):
            plan.spmv_host(hx[0], hy[0], kernel=kernel)
        ks = max(10, min(K, 200))
        t0 = time.perf_counter()
        for _ in range(ks):
            plan.spmv_host(hx[0], hy[0], kernel=kernel)
        sync_s = (time.perf_counter() - t0) / ks
        sync_call = {"value": B / sync_s / 1e9, "ms_per_step": sync_s * 1e3,
                     "rel_err": oracle.rel_errors(hy[0], ydd)[0],
                     "call": "fl_plan_spmv_host (synchronous: one step's latency)"}

    peak, peak_kind = measured_peaks()
    comparators = (measure_comparators(fl, c, x, ydd, B) if (rank == 0 and not args.quick and not args.no_compare)
                   else None)
    forms = measure_forms(fl, peak) if (rank == 0 and not args.quick and not args.no_forms) else None
    batch = measure_batch(fl, peak) if (rank == 0 and not args.quick and not args.no_forms) else None
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = cpu_baseline_sample(c, budget_s=1.0 if args.quick else 12.0) if world == 1 else None
    kname = "k_spmv_form<double,1,1,1,double,1,0>" if plan.info["heavy_cols"] else "k_spmv_stream_f64"
    traffic = ncu_traffic(kname, workload_name(n))
    plan.check()
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": DATA,
        "config": bench_config(c, world),
        "plan": {"kernel": "bucketed (auto)" if plan.info["heavy_cols"] else "stream (auto)",
                 "heavy_band_cols": plan.info["heavy_cols"], "heavy_band_nnz": plan.info["heavy_nnz"],
                 "tilenum": plan.info["tilenum"], "steps_h_count": plan.info["steps"]},
        "pct_of_peak": 100.0 * value / world / peak,
        "gflops": 2.0 * nnz * world / (ms_step * 1e-3) / 1e9,
        "rel_err_vs_fp64_oracle": {"normwise": rel[0], "max_over_inf": rel[1]},
        "kernel_variants_gbs": variants,
        "speedup_vs_plain_fp64_stream": (variants["stream2"] and achieved / variants["stream2"]) if variants else None,
        "preprocess_s": prep_s,
        "comparators": comparators,
        "forms": forms,
        "batch": batch,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": f"{peak_kind} hbm_gbs",
                     "kernel": kname, "bytes_per_launch": B, "kernel_ms": kern_ms,
                     "kernel_ms_isolated": kern_iso_ms,
                     "timing": "kernel_ms: K back-to-back launches between two events; kernel_ms_isolated: "
                               "one launch between two events after a device sleep (launch enqueued first), "
                               "synchronised, L2 not flushed (inputs > L2)"},
        "cpu_baseline": cpu,
        "e2e": {"value": B / e2e_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": m * 8,
                "ms_per_step": e2e_s * 1e3, "steps": ke,
                "call": "fl_plan_spmv_host_async, pinned host x and y, consecutive steps pipelined; wall clock "
                        "from the first call to the stream synchronisation after the last",
                "rel_err": e2e_rel,
                "sync_call": sync_call},
        "gpu_launches": K * launches_per_step,
        "clocks": clk.summary(wall0, wall2),
    }
    print(json.dumps(line), flush=True)
    plan.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="fastload", choices=["fastload", "reference"])
    ap.add_argument("--cols", type=int, default=N_COLS, help="columns of the Zipf matrix (default 1,048,576)")
    ap.add_argument("--profile", default=None, help="case:values:band:k -- run one kernel for a profiler")
    ap.add_argument("--no-forms", action="store_true", help="skip the storage / multi-RHS form measurements")
    ap.add_argument("--no-compare", action="store_true", help="skip the naive-CSC and cuSPARSE comparator lines")
    ap.add_argument("--quick", action="store_true", help="skip kernel variants and the synchronous host call, "
                                                         "shorten e2e and CPU legs (for profiling runs)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus if args.gpus == 1 else 1))
    if args.profile:
        run_profile(args.profile)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
