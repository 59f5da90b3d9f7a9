#!/usr/bin/env python3
"""Benchmark of the local RBF-FD hot path on one GB300 (or N independent replicas).

Workload (default): 3D Laplacian, N = 4,000,000 points i.i.d. uniform in [0,1]^3 (seeded),
PHS(3) with degree-2 polynomials (10 monomials), k = 30 (40x40 saddle-point systems).
A step is one pass of the hot path over the cloud: k-NN stencils, the weight build
(assembly + solve + scatter into CSR) and one apply of the operator to a field.

  value  : stencils built per second over the whole job (all ranks), device-resident inputs
  e2e    : the same metric through the public API with host inputs and a host result
           (points and field copied in, Laplacian of the field copied out, every step)

The headline build is the learned + FP32-refined solve: an MLP (trained before the timed
region on 2,000,000 plain-FP64 solver stencils) predicts each stencil's weights from its
scaled offsets, the prediction seeds the FP32-factorised, FP64-refined solve, and stencils
whose refinement does not converge fall back to the FP64 solve.  The plain FP64 build and
the unseeded refined build are timed beside it, and the max row-relative weight difference
against the plain FP64 weights is reported (equal-error requirement: <= 1e-8).
`--impl reference` times the CPU oracle (a C restatement of the reference algorithm: grid
kNN + raw-coordinate assembly + rook Bunch-Kaufman, OpenMP on all host cores) on a bounded
sample of the same workload.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "stencils/s built (learned+FP32-refined vs plain FP64, equal err); apply GB/s"

CONFIGS = {
    # name: (dim, N, phs, poly_deg, k, ops, field description)
    "lap3d_4M": dict(dim=3, n=4_000_000, phs=3, deg=2, k=30, ops=[(3, 0)], dist="uniform", learned=True,
                     desc="3D Laplacian, N=4,000,000 uniform in [0,1]^3, PHS3 deg 2, k=30 (40x40 systems); "
                          "learned seed: MLP 90->256->256->256->30 GELU, bf16/FP32-acc, trained on 2,000,000 "
                          "solver stencils (uniform + linear +/-20% density-gradient clouds)"),
    "lap2d_10k": dict(dim=2, n=10_000, phs=3, deg=2, k=20, ops=[(3, 0)], dist="uniform",
                      desc="2D Laplacian, N=10,000 uniform in [0,1]^2, PHS3 deg 2, k=20 (26x26 systems)"),
    "gradlap3d_1M": dict(dim=3, n=1_000_000, phs=5, deg=2, k=40, ops=[(1, 0), (1, 1), (1, 2), (3, 0)],
                         dist="lattice", desc="3D gradient+Laplacian, 100^3 jittered lattice, PHS5 deg 2, k=40"),
}


PEAKS = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
    os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}

# DRAM bytes (read + write) per stencil of the headline build kernel: constants from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the same kernel on a 1,000,000-point
# case of this workload (`python bench.py --case build_refined --n 1000000` and `--case
# build_learned` under ncu), scaled by the stencil count (the kernel's traffic grows in
# proportion).  None: not captured.
KERNEL_TRAFFIC_PER_STENCIL = {"fp32_refined": 477.4, "learned": 610.3}


def peaks_bf16():
    return PEAKS.get("bf16_tflops", 1900.0)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="lap3d_4M", choices=sorted(CONFIGS))
    p.add_argument("--n", type=int, default=0, help="override the point count (development runs)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--interp-n", type=int, default=10_000, help="points of the Interpolator leg (0: skip)")
    p.add_argument("--all-configs", action="store_true",
                   help="time the other workloads (2D 10k, 3D gradient+Laplacian 1M, 2D disk Hermite 2M, "
                        "3D regrid 8M) on one GPU, one JSON line each, and exit")
    p.add_argument("--cpu-sample", type=int, default=0, help="stencils in the CPU baseline sample")
    p.add_argument("--train-stencils", type=int, default=2_000_000, help="solver stencils the surrogate trains on")
    p.add_argument("--train-epochs", type=int, default=12)
    p.add_argument("--no-learned", action="store_true", help="headline without the learned seed")
    p.add_argument("--reorder", action="store_true",
                   help="with --profile-once: put the cloud in Morton order first (reorder_points)")
    p.add_argument("--case", default=None, choices=sorted(CASES),
                   help="run one kernel on a small case of the workload (--n points, 1,000,000 by default), "
                        "once to warm up and --reps more times, and exit: the command to capture under ncu")
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--profile-once", action="store_true",
                   help="run each hot kernel once (kNN, FP64 build, FP32-refined build, apply) and exit "
                        "(a short command to capture under ncu)")
    return p.parse_args()


CASES = {
    "knn": "rbf_knn on the cloud (knn_fast_kernel)",
    "build_fp64": "plain FP64 weight build (build_fp64_kernel)",
    "build_refined": "FP32-factorised FP64-refined build (build_refined_split_kernel<40> + build_deferred_kernel)",
    "build_learned": "learned + refined build (features, tcgen05 inference, seeded split-row kernel)",
    "features": "surrogate inputs (features_kernel)",
    "mlp_infer": "surrogate inference, four tcgen05 GEMMs (gemm_tc_persistent_kernel)",
    "mlp_train": "surrogate training steps, batch 4096 (gemm_bf16_kernel and the Adam / loss kernels)",
    "spmv_sell": "single-field apply of the built operator, sliced-ELL copy (spmv_sell_kernel)",
    "spmv_csr": "single-field apply of the built operator, CSR (spmv_pair_kernel)",
    "spmm16": "16-field apply of the built operator, column-major fields (spmm_interleaved_kernel)",
    "spmv_ordered": "single-field apply, sliced copy in the points' Morton order, x and y in the caller's order "
                    "(gather_perm_kernel + spmv_sell_perm_kernel)",
    "step": "one headline step: kNN + features + tcgen05 inference + seeded refined build (CSR + sliced copy) + "
            "one apply (an untrained surrogate: the same kernels as a trained one)",
}


def run_case(args, pkg, ctx, torch, dev):
    """One kernel of the headline workload on a small cloud: set-up, one warm-up call, then
    args.reps calls of the kernel named by args.case (for ncu -k ... -s ... -c ...)."""
    cfg = CONFIGS[args.config]
    n = args.n or 1_000_000
    X_h = make_points(cfg, n, 1000)
    if args.reorder:
        X_h = X_h[np.lexsort(np.floor(X_h * 64).T[::-1])]  # cell-sorted points (locality)
    Xd = torch.from_numpy(X_h).to(dev)
    k = cfg["k"]
    basis = pkg.PHS(cfg["phs"], poly_deg=cfg["deg"])
    case = args.case
    from importlib import import_module
    L = import_module(pkg.__name__ + ".learned")
    adjl = pkg.find_neighbors(Xd, k=k, ctx=ctx) if case not in ("knn", "step") else None
    model = None
    if case == "build_learned":  # a trained surrogate: its seed decides the refinement's path
        Xb, T = L.training_set(100_000, 100_000, k, cfg["dim"], basis, cfg["ops"], seed=5000, ctx=ctx)
        model, _ = L.train_surrogate(Xb, T, k, cfg["dim"], epochs=3, batch=4096, ctx=ctx)
    elif case in ("features", "mlp_infer", "mlp_train", "step"):  # the kernels' work does not depend on the weights
        model = L.StencilMLP(k, cfg["dim"], ctx=ctx, seed=0)
    W = None
    if case.startswith("spm"):
        W = pkg.build_weights(cfg["ops"], Xd, None, adjl, basis, precision="fp32_refined", ctx=ctx,
                              sell=case == "spmv_sell")[-1]
        if case == "spmv_csr":
            W.sell = None
        if case == "spmv_ordered":
            W = W.to_sell_ordered(Xd)
    f = torch.from_numpy(np.sin(4 * X_h[:, 0]) * np.cos(3 * X_h[:, 1])).to(dev)
    F16 = torch.randn((16, n), dtype=torch.float64, device=dev) if case == "spmm16" else None
    feats = model.features(Xd, None, adjl) if case == "mlp_infer" else None
    if case == "mlp_train":
        Xt = model.features(Xd, None, adjl[:4096])
        Tt = torch.zeros((4096, model.dims[-1]), dtype=torch.float32, device=dev)
        Tt[:, :k] = torch.randn((4096, k), dtype=torch.float32, device=dev)
    st = pkg._native.BuildStats()
    fns = {
        "knn": lambda: pkg.find_neighbors(Xd, k=k, ctx=ctx),
        "build_fp64": lambda: pkg.build_weights(cfg["ops"], Xd, None, adjl, basis, precision="fp64", ctx=ctx, stats=st),
        "build_refined": lambda: pkg.build_weights(cfg["ops"], Xd, None, adjl, basis, precision="fp32_refined",
                                                   ctx=ctx, stats=st),
        "build_learned": lambda: L.build_learned(model, cfg["ops"], Xd, adjl, basis, ctx=ctx, stats=st),
        "features": lambda: model.features(Xd, None, adjl),
        "mlp_infer": lambda: model.predict(feats),
        "mlp_train": lambda: model.train_step(Xt, Tt, lr=1e-3),
        "spmv_sell": lambda: W.apply(f),
        "spmv_csr": lambda: W.apply(f),
        "spmm16": lambda: W.apply(F16.T),
        "spmv_ordered": lambda: W.apply(f),
        "step": lambda: L.build_learned(model, cfg["ops"], Xd, pkg.find_neighbors(Xd, k=k, ctx=ctx), basis, ctx=ctx,
                                        sell=True)[-1].apply(f),
    }
    fn = fns[case]
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream()
    e0.record(stream)
    for _ in range(args.reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    print(json.dumps({"case": case, "what": CASES[case], "n": n, "reps": args.reps,
                      "ms_per_call": e0.elapsed_time(e1) / args.reps, "ms_build": float(st.ms_build),
                      "note": "a development timing, not a bench value"}), flush=True)


def make_points(cfg, n, seed, torch=None, device=None):
    rng = np.random.default_rng(seed)
    if cfg["dist"] == "uniform":
        X = rng.uniform(0.0, 1.0, (n, cfg["dim"]))
    else:
        m = round(n ** (1.0 / cfg["dim"]))
        g = np.stack(np.meshgrid(*[np.arange(m)] * cfg["dim"], indexing="ij"), -1).reshape(-1, cfg["dim"])
        X = (g + 0.5 + rng.uniform(-0.3, 0.3, g.shape)) / m
    return X


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def row_rel_err_torch(torch, row_ptr, k, v, vref):
    ne = row_ptr.numel() - 1
    d = (v - vref).abs().reshape(ne, k).amax(1)
    s = vref.abs().reshape(ne, k).amax(1).clamp_min(1e-300)
    return float((d / s).max())


def cpu_baseline(cfg, n, sample, X=None, seed=1000):
    """The oracle (C restatement of the reference algorithm) on host cores, bounded sample: the
    grid kNN of the first `sample` points over the whole cloud and their weights.  X: the
    cloud the GPU builds (the same seeded cloud is made here otherwise).  Returns the timing
    and the oracle's CSR of those rows."""
    from oracle import oracle as O
    if X is None:
        X = make_points(cfg, n, seed)
    q = X[:sample]
    t0 = time.perf_counter()
    adjl = O.knn(X, q, cfg["k"])
    t1 = time.perf_counter()
    ref = O.build(X, q, adjl, cfg["dim"], cfg["phs"], cfg["deg"], cfg["ops"])
    t2 = time.perf_counter()
    return {"stencils_per_s": sample / (t2 - t0), "knn_s": t1 - t0, "build_s": t2 - t1,
            "cores": O.num_threads(), "sample": sample, "ref": ref, "adjl": adjl}


def oracle_errors(torch, W, ref, f, op_index=0):
    """A GPU operator's first rows against the oracle's weights of the same stencils: max and RMS
    of the row-relative weight difference (row max-norm), and the relative max difference of
    the operator applied to the test function f (numpy, all data points)."""
    from oracle import oracle as O
    ne = len(ref.row_ptr) - 1
    m = int(ref.row_ptr[-1])
    rp = W.row_ptr[: ne + 1].cpu().numpy()
    if not np.array_equal(rp, ref.row_ptr) or not np.array_equal(W.col[:m].cpu().numpy(), ref.col):
        return {"structure_equal": False}
    v = W.val[:m].cpu().numpy()
    vr = ref.val[op_index]
    rows = np.repeat(np.arange(ne), np.diff(ref.row_ptr))
    num, den = np.zeros(ne), np.zeros(ne)
    np.maximum.at(num, rows, np.abs(v - vr))
    np.maximum.at(den, rows, np.abs(vr))
    ok = den > 0
    rel = num[ok] / den[ok]
    y = np.zeros(ne)
    np.add.at(y, rows, v * f[ref.col])
    yr = O.spmm(ref, f, op_index)
    return {"structure_equal": True, "max_row_rel_weight_err": float(rel.max()),
            "rms_row_rel_weight_err": float(np.sqrt((rel ** 2).mean())),
            "operator_on_test_function_rel_err": float(np.abs(y - yr).max() / np.abs(yr).max())}


def max_over_ranks(ms, world, device=None):
    """The job's time: the slowest rank's (every rank passes its own; a no-op on one rank)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, ms):
    """Whole-job throughput: the units all ranks processed over the slowest rank's time
    (replicas: every rank processes its own cloud of the same size)."""
    return units_per_rank * world / (ms * 1e-3)


def halton(n, base):
    """Radical-inverse sequence of base `base`, indices 1..n."""
    out = np.zeros(n)
    idx = np.arange(1, n + 1)
    f = 1.0
    while idx.any():
        f /= base
        out += f * (idx % base)
        idx //= base
    return out


def franke(p):
    x, y = p[:, 0], p[:, 1]
    return (0.75 * np.exp(-(9 * x - 2) ** 2 / 4 - (9 * y - 2) ** 2 / 4)
            + 0.75 * np.exp(-(9 * x + 1) ** 2 / 49 - (9 * y + 1) / 10)
            + 0.5 * np.exp(-(9 * x - 7) ** 2 / 4 - (9 * y - 3) ** 2 / 4)
            - 0.2 * np.exp(-(9 * x - 4) ** 2 - (9 * y - 7) ** 2))


def interp_bench(pkg, torch, stream, n_points, cpu):
    """Interpolator on Franke's function at Halton points (the reference's interpolation
    test, PHS3 degree 2) at n_points: fit (assembly + rook Bunch-Kaufman + solve) and the
    evaluation at 1M points, on the GPU; LAPACK's dsytrf_rook (all host cores) and the oracle's
    evaluation beside it."""
    x = np.stack([halton(n_points, 2), halton(n_points, 3)], 1)
    y = franke(x)
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    basis = pkg.PHS(3, poly_deg=2)
    I = pkg.Interpolator(xd, yd, basis)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    reps = 2
    for _ in range(reps):
        I = pkg.Interpolator(xd, yd, basis)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_fit = e0.elapsed_time(e1) / reps
    m = 1_000_000
    xe = torch.rand((m, 2), dtype=torch.float64, device=xd.device, generator=torch.Generator(device=xd.device).manual_seed(3))
    I(xe)
    torch.cuda.synchronize()
    e0.record(stream)
    v = I(xe)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_eval = e0.elapsed_time(e1)
    err = float(np.abs(v.cpu().numpy() - franke(xe.cpu().numpy())).max())
    nt = n_points + 6
    fl = nt ** 3 / 3.0  # symmetric indefinite factorisation
    by = 16.0 * nt ** 3 / 6.0  # unblocked updates: each leading-triangle entry read and written per step
    out = {"workload": f"Franke's function on {n_points} Halton points, PHS3 degree 2 (n = {nt}); eval at {m} points",
           "fit_ms": ms_fit, "eval_ms": ms_eval, "eval_points_per_s": m / (ms_eval * 1e-3),
           "eval_pairs_per_s": m * n_points / (ms_eval * 1e-3), "max_abs_err_vs_franke": err,
           "factor_fp64_tflops": fl / (ms_fit * 1e-3) / 1e12,
           "factor_update_gbs": by / (ms_fit * 1e-3) / 1e9,
           "kernels": "interp_assemble_kernel, rook_step_kernel per column (unblocked "
                      "dsytf2_rook order), blocked solve, interp_eval_kernel"}
    if cpu:
        from oracle import oracle as O
        solver = O.lapack_rook_solver()
        if solver is not None:
            t0 = time.perf_counter()
            w = O.interp_fit(x, y, 3, 2, solver=solver)
            t1 = time.perf_counter()
            me = 20_000
            O.interp_eval(x, w, xe[:me].cpu().numpy(), 3, 2)
            t2 = time.perf_counter()
            out["cpu"] = {"fit_ms": (t1 - t0) * 1e3, "kind": "reference LAPACK (OpenBLAS dsytrf_rook, the routine "
                          "bunchkaufman! calls) + oracle assembly", "cores": O.num_threads(),
                          "eval_points_per_s": me / (t2 - t1), "eval_sample": me}
    return out


def unit_disk(n_interior, n_boundary, seed):
    """Jittered grid clipped to the open unit disk plus equispaced boundary points with outward
    normals; Dirichlet on the upper half-circle, Neumann on the lower."""
    rng = np.random.default_rng(seed)
    m = int(math.sqrt(n_interior * 4 / math.pi))
    h = 2.0 / m
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 2)
    P = -1 + (g + 0.5) * h + rng.uniform(-0.3 * h, 0.3 * h, g.shape)
    P = P[np.hypot(P[:, 0], P[:, 1]) < 1 - 0.5 * h]
    t = 2 * math.pi * (np.arange(n_boundary) + 0.5) / n_boundary
    B = np.stack([np.cos(t), np.sin(t)], 1)
    isb = np.zeros(len(P) + n_boundary, dtype=bool)
    isb[len(P):] = True
    dirichlet = B[:, 1] > 0
    return np.concatenate([P, B]), isb, B, np.where(dirichlet, 1.0, 0.0), np.where(dirichlet, 0.0, 1.0)


def mixture_targets(n, seed):
    """Half uniform in the unit cube, half from 8 isotropic Gaussians (sigma 0.05), clipped."""
    rng = np.random.default_rng(seed)
    half = n // 2
    centres = rng.uniform(0.1, 0.9, (8, 3))
    G = centres[rng.integers(0, 8, n - half)] + rng.normal(0, 0.05, (n - half, 3))
    return np.clip(np.concatenate([rng.uniform(0, 1, (half, 3)), G]), 0.0, 1.0)


def fourier_fields(torch, X, nf, seed):
    """nf seeded smooth fields, each a sum of 8 Fourier modes (wavenumbers uniform in [1, 4] per
    axis, N(0, 1) amplitudes), as an (n, nf) tensor on X's device."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    kv = torch.rand((nf, 8, X.shape[1]), generator=g, dtype=torch.float64) * 3 + 1
    a = torch.randn((nf, 8), generator=g, dtype=torch.float64)
    F = torch.empty((X.shape[0], nf), dtype=torch.float64, device=X.device)
    for f in range(nf):
        F[:, f] = (torch.sin(X @ kv[f].T.to(X.device)) * a[f].to(X.device)).sum(1)
    return F


def all_configs(pkg, torch, ctx, stream, cpu=True):
    """The other workloads of the benchmark's configuration list, each timed once on the GPU:
    kNN, plain FP64, FP32-refined and (3D regrid) learned + refined builds (stencils/s, build
    only), every build's max / RMS row-relative weight error and operator-on-test-function error
    against the oracle (the reference algorithm on the host, on a sample of the same stencils:
    the whole cloud where it is small or has Hermite rows), and the apply (algorithmic bytes over
    the library's kernel time, fraction of the measured copy rate or of the FP64 FMA rate).  One
    JSON line per workload."""
    from importlib import import_module
    from oracle import oracle as O
    L = import_module(pkg.__name__ + ".learned")
    hbm = PEAKS.get("hbm_gbs", 6800.0)

    def ev_ms(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, out

    def kernel_ms(fn):
        ctx.lib.rbf_ctx_set_timing(ctx.h, 1)
        fn()
        fn()
        v = pkg.ctypes.c_float(0.0)
        ctx.lib.rbf_ctx_last_ms(ctx.h, pkg.ctypes.byref(v))
        ctx.lib.rbf_ctx_set_timing(ctx.h, 0)
        return float(v.value)

    fma64 = pkg.ctypes.c_double(0.0)
    ctx.check(ctx.lib.rbf_diag_fma_peak(ctx.h, 1, pkg.ctypes.byref(fma64)))
    fma_peak = fma64.value / 2.0  # FP64 FMA per second (the peak counts 2 flops per FMA), in T

    def vs_oracle(Ws, ref, f):
        """Worst over the operators of oracle_errors on the sampled rows; ref is a pair (the
        reference arithmetic's weights, the local-frame oracle's) or None."""
        if ref is None:
            return None
        if isinstance(ref, tuple):
            return {"reference_arithmetic": vs_oracle(Ws, ref[0], f), "local_frame": vs_oracle(Ws, ref[1], f)}
        errs = [oracle_errors(torch, W, ref, f, q) for q, W in enumerate(Ws)]
        if not all(e.get("structure_equal") for e in errs):
            return {"structure_equal": False}
        return {"structure_equal": True,
                "max_row_rel_weight_err": max(e["max_row_rel_weight_err"] for e in errs),
                "rms_row_rel_weight_err": max(e["rms_row_rel_weight_err"] for e in errs),
                "operator_on_test_function_rel_err": max(e["operator_on_test_function_rel_err"] for e in errs)}

    def report(name, desc, ne, ms_knn, builds, ref_info, W, nf, ms_apply, extra=None):
        by = W.nnz * 12 + (ne + 1) * 8 + nf * (W.shape[1] + ne) * 8
        fmas = W.nnz * nf / (ms_apply * 1e-3) / 1e12
        ms64 = builds["fp64"]["ms_build"]
        for b in builds.values():
            b["stencils_per_s"] = ne / (b["ms_build"] * 1e-3)
            b["speedup_vs_fp64"] = ms64 / b["ms_build"]
        line = {"workload": name, "desc": desc, "stencils": ne, "ms_knn": ms_knn, "builds": builds,
                "oracle_sample": ref_info, "bar": 1e-8,
                "oracle_frames": "reference_arithmetic: the reference's algorithm in its raw coordinates; "
                                 "local_frame: the same formulation assembled per stencil centred at the eval "
                                 "point and scaled by a power of two (pinned to 60-digit truth where the raw "
                                 "systems are ill-conditioned)",
                "apply": {"fields": nf, "nnz": W.nnz, "ms": ms_apply, "GB_s": by / (ms_apply * 1e-3) / 1e9,
                          "frac_of_hbm": by / (ms_apply * 1e-3) / 1e9 / hbm,
                          "fp64_fma_T_per_s": fmas, "frac_of_fp64_fma": fmas / fma_peak,
                          "bound": "hbm" if by / (W.nnz * nf) > hbm / (fma_peak * 1e3) else "fp64 FMA (nnz x fields)"}}
        if extra:
            line.update(extra)
        print(json.dumps(line), flush=True)

    def aug_errors(W, rows, rp, col, val, f):
        """GPU rows `rows` of a normal-derivative build against the oracle's (rp, col, val):
        structure, max / RMS row-relative weight error, and the rows applied to f = [u; du/dn]."""
        grp, gcol, gval = W.row_ptr.cpu().numpy(), W.col.cpu().numpy(), W.val.cpu().numpy()
        rel, y, yr = [], [], []
        for t, e in enumerate(rows):
            c, v = gcol[grp[e]:grp[e + 1]], gval[grp[e]:grp[e + 1]]
            cr, vr = col[rp[t]:rp[t + 1]], val[rp[t]:rp[t + 1]]
            if not np.array_equal(c, cr):
                return {"structure_equal": False}
            rel.append(np.abs(v - vr).max() / np.abs(vr).max())
            y.append(v @ f[c])
            yr.append(vr @ f[cr])
        rel, y, yr = np.array(rel), np.array(y), np.array(yr)
        return {"structure_equal": True, "max_row_rel_weight_err": float(rel.max()),
                "rms_row_rel_weight_err": float(np.sqrt((rel ** 2).mean())),
                "operator_on_test_function_rel_err": float(np.abs(y - yr).max() / np.abs(yr).max())}

    def stats_of(st):
        return {"fallback_stencils": int(st.n_fallback),
                "residuals_per_stencil": float(st.n_residuals) / max(1, int(st.n_stencils))}

    dev = torch.device("cuda", ctx.device)
    # ---- C1: 2D Laplacian, 10,000 uniform points, PHS3 degree 2, k = 20 (oracle: every stencil)
    rng = np.random.default_rng(101)
    Xh = rng.uniform(0, 1, (10_000, 2))
    X = torch.from_numpy(Xh).to(dev)
    ms_knn, a = ev_ms(lambda: pkg.find_neighbors(X, k=20, ctx=ctx))
    b = pkg.PHS(3, poly_deg=2)
    ms64, W64 = ev_ms(lambda: pkg.build_weights([(3, 0)], X, None, a, b, ctx=ctx)[0])
    st = pkg._native.BuildStats()
    ms32, W32 = ev_ms(lambda: pkg.build_weights([(3, 0)], X, None, a, b, ctx=ctx, precision="fp32_refined",
                                                stats=st)[0])
    f = np.sin(4 * Xh[:, 0]) * np.cos(3 * Xh[:, 1])
    ref = tuple(O.build(Xh, Xh, a.cpu().numpy(), 2, 3, 2, [(3, 0)], frame=fr) for fr in ("raw", "local")) \
        if cpu else None
    builds = {"fp64": {"ms_build": ms64, "vs_oracle": vs_oracle([W64], ref, f)},
              "fp32_refined": {"ms_build": ms32, "vs_oracle": vs_oracle([W32], ref, f), **stats_of(st)}}
    fd = torch.from_numpy(f).to(dev)
    lap = W32.apply(fd)
    inner = ((X > 0.1) & (X < 0.9)).all(1)
    err_f = float(((lap + 25 * fd)[inner]).abs().max() / (25 * fd[inner]).abs().max())
    report("lap2d_10k", "2D Laplacian, 10,000 uniform points, PHS3 degree 2, k = 20 (26 x 26)", 10_000, ms_knn,
           builds, "all 10,000 stencils", W32, 1, kernel_ms(lambda: W32.apply(fd)),
           {"laplacian_rel_err_vs_analytic_interior": err_f, "note": "L2-resident sizes: launch-bound, not a roofline case"})
    # ---- C2: 3D gradient + Laplacian, 100^3 jittered lattice, PHS5 degree 2, k = 40, 16 fields
    cfg = CONFIGS["gradlap3d_1M"]
    Xh = make_points(cfg, 1_000_000, 102)
    X = torch.from_numpy(Xh).to(dev)
    ms_knn, a = ev_ms(lambda: pkg.find_neighbors(X, k=40, ctx=ctx))
    b = pkg.PHS(5, poly_deg=2)
    ms64, W64 = ev_ms(lambda: pkg.build_weights(cfg["ops"], X, None, a, b, ctx=ctx))
    st = pkg._native.BuildStats()
    ms32, W32 = ev_ms(lambda: pkg.build_weights(cfg["ops"], X, None, a, b, ctx=ctx, precision="fp32_refined",
                                                stats=st))
    m = 100_000
    f = np.sin(2 * Xh[:, 0]) * np.cos(3 * Xh[:, 1]) * np.exp(Xh[:, 2])
    ref = tuple(O.build(Xh, Xh[:m], a[:m].cpu().numpy(), 3, 5, 2, cfg["ops"], frame=fr) for fr in ("raw", "local")) \
        if cpu else None
    builds = {"fp64": {"ms_build": ms64, "vs_oracle": vs_oracle(W64, ref, f)},
              "fp32_refined": {"ms_build": ms32, "vs_oracle": vs_oracle(W32, ref, f), **stats_of(st)}}
    F = fourier_fields(torch, X, 16, 103)
    report("gradlap3d_1M", "3D gradient + Laplacian (4 operators, one factorisation), 100^3 jittered lattice, "
           "PHS5 degree 2, k = 40 (50 x 50); 16 fields per operator", 1_000_000, ms_knn, builds,
           f"first {m} stencils", W32[3], 16, kernel_ms(lambda: W32[3].apply(F)))
    del W64, W32, F, a, X
    # ---- C3: 2D unit disk, 2,000,000 interior + 5,000 boundary points, Dirichlet / Neumann, PHS3 degree 3, k = 30
    Xh, isb, nrm, al, be = unit_disk(2_000_000, 5_000, 104)
    X = torch.from_numpy(Xh).to(dev)
    ms_knn, a = ev_ms(lambda: pkg.find_neighbors(X, k=30, ctx=ctx))
    herm = dict(is_boundary=isb, bc=[pkg.BoundaryCondition(x, y) for x, y in zip(al, be)], normals=nrm)
    ap, ai = pkg.ragged_stencils(a, torch.full((len(Xh),), 30, device=dev))
    b = pkg.PHS(3, poly_deg=3)
    st = pkg._native.BuildStats()
    run = lambda prec: pkg.build_weights_batched([(3, 0)], X, None, ap, ai, b, hermite=herm, precision=prec,
                                                 tune=1, ctx=ctx, stats=st)[0]
    ms64, W64 = ev_ms(lambda: run("fp64"))
    s64 = stats_of(st)
    ms32, W32 = ev_ms(lambda: run("fp32_refined"))
    s32 = stats_of(st)
    u = Xh[:, 0] ** 2 + Xh[:, 1] ** 2 + 1.0
    ref = tuple(O.build(Xh, Xh, a.cpu().numpy(), 2, 3, 3, [(3, 0)], hermite=(isb.astype(np.uint8), al, be, nrm),
                        frame=fr) for fr in ("raw", "local")) if cpu else None
    builds = {"fp64": {"ms_build": ms64, "vs_oracle": vs_oracle([W64], ref, u)},
              "fp32_refined": {"ms_build": ms32, "vs_oracle": vs_oracle([W32], ref, u), **s32}}
    ud = torch.from_numpy(u).to(dev)
    report("disk_hermite_2M", f"2D unit disk, {len(Xh) - 5000} interior + 5,000 boundary points (Dirichlet upper, "
           "Neumann lower half-circle), PHS3 degree 3, k = 30 (40 x 40, Hermite rows on boundary stencils), one "
           "persistent batched launch with autotuned tiles", len(Xh), ms_knn, builds, "all stencils", W32, 1,
           kernel_ms(lambda: W32.apply(ud)))
    # the same disk with du/dn unknowns at the Neumann points (RBF_FLAG_NORMAL_DOF): boundary-
    # adjacent stencils solve 40 + m systems, m their Neumann neighbours, all in one launch
    nd_run = lambda prec: pkg.build_weights_batched([(3, 0)], X, None, ap, ai, b, hermite=herm, precision=prec,
                                                    tune=1, ctx=ctx, stats=st, normal_dof=True)[0]
    ms64, W64 = ev_ms(lambda: nd_run("fp64"))
    ms32, W32 = ev_ms(lambda: nd_run("fp32_refined"))
    s32 = stats_of(st)
    ah = a.cpu().numpy()
    bidx = np.nonzero(isb)[0]
    nr_pt = np.zeros(len(Xh), bool)
    nr_pt[bidx[be != 0.0]] = True
    dir_pt = np.zeros(len(Xh), bool)
    dir_pt[bidx[be == 0.0]] = True
    m_of = np.where(dir_pt, 0, nr_pt[ah].sum(1))
    sizes = np.bincount(30 + 10 + m_of[~dir_pt])
    builds = {"fp64": {"ms_build": ms64}, "fp32_refined": {"ms_build": ms32, **s32}}
    if cpu:
        from oracle import augmented_oracle as A
        rows = np.concatenate([np.nonzero(m_of > 0)[0][::3][:1500], np.nonzero((m_of == 0) & ~dir_pt)[0][:500]])
        rp, col, val = A.build_augmented(Xh, ah, 2, 3, 3, [(3, 0)], (isb, al, be, nrm), rows=rows)
        dudn = (2.0 * Xh[bidx] * nrm).sum(1)
        fa = np.concatenate([u, dudn])
        for nm, Wx in (("fp64", W64), ("fp32_refined", W32)):
            builds[nm]["vs_oracle"] = {"normal_dof_oracle": aug_errors(Wx, rows, rp, col, val[0], fa)}
    report("disk_hermite_normal_dof_2M", f"the 2D unit disk above with u and du/dn unknowns at the Neumann points "
           "(Hermite-Birkhoff stencils, RBF_FLAG_NORMAL_DOF): boundary-adjacent systems of 40 + m, m the stencil's "
           "Neumann neighbours, all sizes in one persistent launch", len(Xh), ms_knn, builds,
           "1,500 stencils with Neumann neighbours and 500 interior ones (oracle/augmented_oracle.py)", W32, 1,
           kernel_ms(lambda: W32.apply(torch.from_numpy(np.concatenate([u, np.zeros(len(bidx))])).to(dev))),
           {"system_sizes": {int(n): int(c) for n, c in enumerate(sizes) if c}})
    del W64, W32, a, ap, ai, X
    # ---- C5: 3D regrid, 8,000,000 uniform sources onto 8,000,000 mixture targets, PHS3 degree 1, k = 20,
    # 32 fields; the learned form with a surrogate trained on 2,000,000 regrid stencils
    rng = np.random.default_rng(105)
    Sh = rng.uniform(0, 1, (8_000_000, 3))
    Th = mixture_targets(8_000_000, 106)
    S = torch.from_numpy(Sh).to(dev)
    T = torch.from_numpy(Th).to(dev)
    ms_knn, a = ev_ms(lambda: pkg.find_neighbors(S, T, k=20, ctx=ctx), reps=1)
    b = pkg.PHS(3, poly_deg=1)
    t0 = time.perf_counter()
    Xb, Tt = L.training_set(1_000_000, 1_000_000, 20, 3, b, [(0, 0)], seed=6000, ctx=ctx, separate_eval=True)
    model, hist = L.train_surrogate(Xb, Tt, 20, 3, epochs=8, batch=4096, lr=2e-3, ctx=ctx)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del Xb, Tt
    ms64, W64 = ev_ms(lambda: pkg.build_weights([(0, 0)], S, T, a, b, ctx=ctx)[0], reps=1)
    st = pkg._native.BuildStats()
    ms32, W32 = ev_ms(lambda: pkg.build_weights([(0, 0)], S, T, a, b, ctx=ctx, precision="fp32_refined",
                                                stats=st)[0], reps=1)
    s32 = stats_of(st)
    stl = pkg._native.BuildStats()
    msl, Wl = ev_ms(lambda: L.build_learned(model, [(0, 0)], S, a, b, ctx=ctx, stats=stl, eval_points=T)[0], reps=1)
    sl = stats_of(stl)
    sl["seed_rel_err_mean_judged_by_solve"] = float(stl.seed_rel_err_mean)
    m = 200_000
    f = np.sin(3 * Sh[:, 0]) * np.cos(2 * Sh[:, 1]) + Sh[:, 2] ** 2
    ref = tuple(O.build(Sh, Th[:m], a[:m].cpu().numpy(), 3, 3, 1, [(0, 0)], frame=fr) for fr in ("raw", "local")) \
        if cpu else None
    builds = {"fp64": {"ms_build": ms64, "vs_oracle": vs_oracle([W64], ref, f)},
              "fp32_refined": {"ms_build": ms32, "vs_oracle": vs_oracle([W32], ref, f), **s32},
              "learned": {"ms_build": msl, "vs_oracle": vs_oracle([Wl], ref, f), **sl,
                          "note": "features + tcgen05 inference + seeded refined build"}}
    del W64, Wl
    F = fourier_fields(torch, S, 32, 107)
    ms_apply = kernel_ms(lambda: W32.apply(F))
    # the same operator on Morton-ordered sources and targets (reorder_points): the gathers of
    # the 32-field rows become local, so each source row is read from HBM about once
    del W32, a
    ps, So = pkg.reorder_points(S, ctx=ctx)
    pt, To = pkg.reorder_points(T, ctx=ctx)
    ao = pkg.find_neighbors(So, To, k=20, ctx=ctx)
    Wo = pkg.build_weights([(0, 0)], So, To, ao, b, ctx=ctx, precision="fp32_refined")[0]
    Fo = F[ps.long()].contiguous()
    ms_o = kernel_ms(lambda: Wo.apply(Fo))
    by = Wo.nnz * 12 + (8_000_001) * 8 + 32 * 16_000_000 * 8
    report("regrid3d_8M", "3D regrid, 8,000,000 uniform sources onto 8,000,000 targets (50 % uniform, 50 % from 8 "
           "Gaussians), PHS3 degree 1, k = 20 (24 x 24); 32 fields", 8_000_000, ms_knn, builds,
           f"first {m} stencils", Wo, 32, ms_apply,
           {"surrogate": {"train_stencils": 2_000_000, "epochs": 8, "train_s": train_s, "loss_last_epoch": hist[-1],
                          "training_clouds": "uniform and +/-20 % density-gradient sources, independent eval clouds "
                                             "of the same distribution"},
            "apply_morton_order": {"ms": ms_o, "GB_s": by / (ms_o * 1e-3) / 1e9,
                                   "frac_of_hbm": by / (ms_o * 1e-3) / 1e9 / hbm}})


def run_reference(args, cfg, n):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sample = args.cpu_sample or (200_000 if cfg["n"] >= 1_000_000 else n)
    times = []
    res = None
    X = make_points(cfg, n, 1000)  # the cloud rank 0 of the GPU arm builds
    for s in range(args.warmup + args.steps):
        res = cpu_baseline(cfg, n, sample, X=X)
        if s >= args.warmup:
            times.append(sample / res["stencils_per_s"])
    v = sample * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "stencils/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": cfg["desc"], "sample_stencils": sample},
        "cpu_baseline": {"value": v, "unit": "stencils/s", "cores": res["cores"], "kind": "port",
                         "sample": f"the first {sample} stencils of the same seeded {n}-point cloud (kNN over "
                                   "all points + build) per step; value = their rate, the full cloud's time "
                                   "extrapolated from it"},
        "extrapolated_full_step_s": n / v,
        "e2e": {"value": v, "unit": "stencils/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference Julia path: unavailable on this box (no Julia); CPU oracle timed instead",
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    cfg = CONFIGS[args.config]
    n = args.n or cfg["n"]
    if args.impl == "reference":
        run_reference(args, cfg, n)
        return

    import torch
    import torch.distributed as dist
    import __graft_entry__ as g

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    g.build()
    pkg = g.load_package()
    ctx = pkg.Context.default(local)
    stream = torch.cuda.current_stream()  # the package binds the library to this stream
    dev = torch.device("cuda", local)
    if args.all_configs:
        all_configs(pkg, torch, ctx, stream, cpu=not args.no_cpu_baseline)
        return
    if args.case:
        run_case(args, pkg, ctx, torch, dev)
        return

    # independent seeded cloud per rank (weak scaling: per-GPU work fixed)
    X_h = make_points(cfg, n, 1000 + rank)
    Xd = torch.from_numpy(X_h).to(dev)
    f_h = np.sin(4 * X_h[:, 0]) * np.cos(3 * X_h[:, 1]) * (np.exp(X_h[:, 2]) if cfg["dim"] == 3 else 1.0)
    fd = torch.from_numpy(f_h).to(dev)
    basis = pkg.PHS(cfg["phs"], poly_deg=cfg["deg"])
    k = cfg["k"]

    learned_on = bool(cfg.get("learned")) and not args.no_learned and len(cfg["ops"]) == 1
    headline = "learned" if learned_on else "fp32_refined"
    L = None
    model = None
    training = None
    if learned_on:
        from importlib import import_module
        L = import_module(pkg.__name__ + ".learned")

    def build(precision, X, adjl, stats=None, sell=True):
        # the build writes the sliced-ELL copy next to the CSR; single-field applies use it
        if precision == "learned":
            return L.build_learned(model, cfg["ops"], X, adjl, basis, ctx=ctx, stats=stats, sell=sell)
        return pkg.build_weights(cfg["ops"], X, None, adjl, basis, precision=precision, ctx=ctx, stats=stats,
                                 sell=sell)

    def step(precision, X=Xd, f=fd):
        adjl = pkg.find_neighbors(X, k=k, ctx=ctx)
        Ws = build(precision, X, adjl)
        y = Ws[-1].apply(f)
        return adjl, Ws, y

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
            torch.cuda.synchronize()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        barrier()
        return max_over_ranks(e0.elapsed_time(e1) / steps, world, dev)

    if learned_on:
        # ---- surrogate training (untimed): plain FP64 solves on independent seeded clouds,
        # half uniform, half with a linear +/-20% density gradient; held-out uniform stencils
        # measure the surrogate's weight error before and after training
        t0 = time.perf_counter()
        nt = args.train_stencils
        Xb, T = L.training_set(nt // 2, nt - nt // 2, k, cfg["dim"], basis, cfg["ops"], seed=5000 + rank, ctx=ctx)
        Xv, Tv = L.training_set(50_000, 0, k, cfg["dim"], basis, cfg["ops"], seed=9000 + rank, ctx=ctx)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        untrained = L.StencilMLP(k, cfg["dim"], ctx=ctx, seed=0, out_scale=float(T.std()))
        u_max, u_med = L.surrogate_error(untrained, Xv, Tv)
        model, hist = L.train_surrogate(Xb, T, k, cfg["dim"], epochs=args.train_epochs, batch=4096, lr=2e-3, ctx=ctx)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        e_max, e_med = L.surrogate_error(model, Xv, Tv)
        training = {"stencils": nt, "epochs": args.train_epochs, "batch": 4096, "data_s": t1 - t0,
                    "train_s": t2 - t1, "loss_first_epoch": hist[0], "loss_last_epoch": hist[-1],
                    "heldout_row_rel_err_median": {"untrained": u_med, "trained": e_med},
                    "heldout_row_rel_err_max": {"untrained": u_max, "trained": e_max},
                    "dims": model.dims}
        del Xb, T, Xv, Tv, untrained

    if args.profile_once:
        if args.reorder:
            perm, Xd = pkg.reorder_points(Xd, k, ctx=ctx)
            fd = fd[perm.long()].contiguous()
        adjl = pkg.find_neighbors(Xd, k=k, ctx=ctx)
        s64, s32 = pkg._native.BuildStats(), pkg._native.BuildStats()
        W64 = build("fp64", Xd, adjl, s64)
        W32 = build(headline, Xd, adjl, s32)
        W32[-1].apply(fd)
        torch.cuda.synchronize()
        err = max(row_rel_err_torch(torch, a.row_ptr, k, a.val, b.val) for a, b in zip(W32, W64))
        print(json.dumps({"profile_once": cfg["desc"], "n": n, "headline": headline, "ms_build_fp64": s64.ms_build,
                          "ms_build_headline": s32.ms_build, "fallback": s32.n_fallback, "max_diff": err}))
        return
    clocks = ClockSampler(local)
    # ---- headline timed region
    for _ in range(args.warmup):
        step(headline)
    barrier()
    launches0 = ctx.lib.rbf_ctx_kernel_launches(ctx.handle)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step(headline)
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    launches = (ctx.lib.rbf_ctx_kernel_launches(ctx.handle) - launches0) // args.steps
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    value = job_rate(n, world, ms)

    # ---- the same step with the plain FP64 build (and without the learned seed) beside it
    ms_fp64 = timed(lambda: step("fp64"), max(1, args.steps // 2), 1)
    ms_fp32r = timed(lambda: step("fp32_refined"), max(1, args.steps // 2), 1) if learned_on else ms

    # ---- the CPU baseline (untimed for the GPU numbers): the oracle on the first stencils of
    # this cloud; its weights are the reference for the equal-error check below
    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sample = args.cpu_sample or (200_000 if n >= 1_000_000 else n)
        cb = cpu_baseline(cfg, n, sample, X=X_h)
        from oracle import oracle as O
        cb["ref_local"] = O.build(X_h, X_h[:sample], cb["adjl"], cfg["dim"], cfg["phs"], cfg["deg"], cfg["ops"],
                                  frame="local")

    # ---- equal-error check: every GPU build against the oracle's weights of the sampled
    # stencils, and over all stencils against the plain GPU build
    adjl = pkg.find_neighbors(Xd, k=k, ctx=ctx)
    st64 = pkg._native.BuildStats()
    W64 = build("fp64", Xd, adjl, st64)
    st_h = pkg._native.BuildStats()
    W_h = build(headline, Xd, adjl, st_h)
    err = max(row_rel_err_torch(torch, a.row_ptr, k, a.val, b.val) for a, b in zip(W_h, W64))
    rms = max(float(((a.val - b.val) ** 2).mean().sqrt() / (b.val ** 2).mean().sqrt()) for a, b in zip(W_h, W64))
    # operator-on-test-function: both operators applied to the field, relative max difference
    y64, yh = W64[-1].apply(fd), W_h[-1].apply(fd)
    op_err = float((yh - y64).abs().max() / y64.abs().max())
    st32 = st_h
    err32 = err
    W32 = W_h
    if learned_on:
        st32 = pkg._native.BuildStats()
        W32 = build("fp32_refined", Xd, adjl, st32)
        err32 = max(row_rel_err_torch(torch, a.row_ptr, k, a.val, b.val) for a, b in zip(W32, W64))
    vs_oracle = None
    if cb is not None:
        ops_last = len(cfg["ops"]) - 1
        vs_oracle = {"sample_stencils": cb["sample"],
                     "neighbour_lists_equal": bool(np.array_equal(adjl[: cb["sample"]].cpu().numpy(), cb["adjl"])),
                     headline: oracle_errors(torch, W_h[-1], cb["ref"], f_h, ops_last),
                     "fp64": oracle_errors(torch, W64[-1], cb["ref"], f_h, ops_last),
                     "local_frame_oracle": {headline: oracle_errors(torch, W_h[-1], cb["ref_local"], f_h, ops_last),
                                            "fp64": oracle_errors(torch, W64[-1], cb["ref_local"], f_h, ops_last)}}
        if learned_on:
            vs_oracle["fp32_refined"] = oracle_errors(torch, W32[-1], cb["ref"], f_h, ops_last)
            vs_oracle["local_frame_oracle"]["fp32_refined"] = oracle_errors(torch, W32[-1], cb["ref_local"], f_h,
                                                                            ops_last)
    del W64, W_h, W32
    # ---- per-stage timings (device-resident, events on the launching stream)
    ms_b_h = timed(lambda: build(headline, Xd, adjl), 3, 1)
    ms_b_32 = timed(lambda: build("fp32_refined", Xd, adjl), 3, 1) if learned_on else ms_b_h
    ms_b_64 = timed(lambda: build("fp64", Xd, adjl), 2, 1)
    ms_knn = timed(lambda: pkg.find_neighbors(Xd, k=k, ctx=ctx), 3, 1)
    mlp = None
    if learned_on:
        feats = model.features(Xd, None, adjl)
        ms_feat = timed(lambda: model.features(Xd, None, adjl), 3, 1)
        ms_mlp = timed(lambda: model.predict(feats), 3, 1)
        fl = 2 * (model.din * model.dims[1] + sum(a * b for a, b in zip(model.dims[1:-2], model.dims[2:-1]))
                  + model.dims[-2] * model.dout)
        tf = fl * n / (ms_mlp * 1e-3) / 1e12
        mlp = {"ms_features": ms_feat, "ms_forward": ms_mlp, "flops_per_stencil": fl, "tflops": tf,
               "bf16_peak_tflops": peaks_bf16(), "frac_of_bf16_peak": tf / peaks_bf16(),
               "kernel": "gemm_tc_kernel (tcgen05.mma, TMEM accumulators, TMA-fed, 128xBN tiles)"}
        del feats
    def kernel_ms(fn, reps=10):
        """Median device time of the library work inside fn (CUDA events recorded by the
        library around its kernels, rbf_ctx_set_timing)."""
        ctx.lib.rbf_ctx_set_timing(ctx.h, 1)
        fn()
        vals = []
        for _ in range(reps):
            fn()
            v = pkg.ctypes.c_float(0.0)
            ctx.lib.rbf_ctx_last_ms(ctx.h, pkg.ctypes.byref(v))
            vals.append(v.value)
        ctx.lib.rbf_ctx_set_timing(ctx.h, 0)
        return statistics.median(vals)

    W = build(headline, Xd, adjl)[-1]
    ms_spmv_api = timed(lambda: W.apply(fd), 10, 3)
    ms_spmv = kernel_ms(lambda: W.apply(fd))  # sliced-ELL apply
    # the sliced copy in the points' Morton order, x and y in the caller's order (made once,
    # for operators applied many times); its product equals the plain sliced copy's bit for bit
    t0 = time.perf_counter()
    W_ord = W.to_sell_ordered(Xd)
    torch.cuda.synchronize()
    ms_to_ordered = (time.perf_counter() - t0) * 1e3
    ord_equal = bool(torch.equal(W_ord.apply(fd), W.apply(fd)))
    ms_spmv_ord = kernel_ms(lambda: W_ord.apply(fd))
    W_sell, W.sell = W.sell, None
    ms_spmv_csr = kernel_ms(lambda: W.apply(fd))  # the CSR apply of the same operator
    W.sell = W_sell
    ms_knn_kernel = kernel_ms(lambda: pkg.find_neighbors(Xd, k=k, ctx=ctx), 3)
    knn_bytes = 2 * n * cfg["dim"] * 8 + n * k * 4
    nnz = W.nnz
    sell_nnz = int(W.sell.col.shape[0])
    # algorithmic bytes of one apply: val (8 B) + col (4 B) per entry, the row offsets (8 B
    # per row in CSR, per 32-row slice in the sliced copy), the field read once and the
    # result written once
    apply_bytes = sell_nnz * 12 + ((n + 31) // 32 + 1) * 8 + 2 * n * 8
    csr_bytes = nnz * 12 + (n + 1) * 8 + 2 * n * 8
    apply_gbs = apply_bytes / (ms_spmv * 1e-3) / 1e9
    csr_gbs = csr_bytes / (ms_spmv_csr * 1e-3) / 1e9
    ord_gbs = apply_bytes / (ms_spmv_ord * 1e-3) / 1e9
    # operator algebra on the device (a + 2 b over two value arrays of one structure, as a sum of
    # two operators on the same stencils):
    # one entry-wise pass over the value arrays, 24 bytes per entry (two reads, one write)
    alg_out = torch.empty_like(W.val)
    alg_b = W.val.clone()  # a second operand in its own memory
    ms_axpby = kernel_ms(lambda: ctx.check(ctx.lib.rbf_weights_axpby(ctx.h, nnz, 1.0, pkg._ptr(W.val), 2.0,
                                                                      pkg._ptr(alg_b), pkg._ptr(alg_out))))
    ms_axpby_api = timed(lambda: ctx.check(ctx.lib.rbf_weights_axpby(ctx.h, nnz, 1.0, pkg._ptr(W.val), 2.0,
                                                                      pkg._ptr(alg_b), pkg._ptr(alg_out))), 5, 2)
    alg_gbs = 24 * nnz / (ms_axpby * 1e-3) / 1e9
    algebra = {"kernel": "axpby_kernel (rbf_weights_axpby: out = a + 2 b over the values; the scalings are "
                         "powers of two, applied on the integer pipe, so one DADD per entry)", "nnz": nnz,
               "ms": ms_axpby, "ms_per_call_api": ms_axpby_api, "GB_s": alg_gbs,
               "frac_of_hbm": alg_gbs / PEAKS.get("hbm_gbs", 6800.0)}
    del W, W_sell, W_ord, alg_out, alg_b
    hbm_peak = PEAKS.get("hbm_gbs", 6800.0)
    hbm_src = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in PEAKS else "fallback"
    fp64_peak = pkg.ctypes.c_double(0.0)
    ctx.check(ctx.lib.rbf_diag_fma_peak(ctx.h, 1, pkg.ctypes.byref(fp64_peak)))
    fp32_peak = pkg.ctypes.c_double(0.0)
    ctx.check(ctx.lib.rbf_diag_fma_peak(ctx.h, 0, pkg.ctypes.byref(fp32_peak)))
    # the algebra's other bound: one FP64 add per entry at the FP64 pipe's rate (the FMA loop's
    # rate; the peak counts two flops per FMA)
    algebra["fp64_issue_bound_ms"] = nnz / (fp64_peak.value * 0.5e12) * 1e3
    algebra["hbm_bound_ms"] = 24 * nnz / (hbm_peak * 1e9) * 1e3
    nsys = k + math.comb(cfg["deg"] + cfg["dim"], cfg["dim"])
    R = len(cfg["ops"])
    # algorithmic FLOPs of the reference algorithm per stencil: symmetric factor n^3/3,
    # solve 2 n^2 R, assembly ~10 flops per phi / L(phi) evaluation
    flops_stencil = nsys ** 3 / 3 + 2 * nsys ** 2 * R + 10 * (k * (k + 1) / 2 + R * k)
    ms_kernel = float(st_h.ms_build)
    ach = flops_stencil * n / (ms_kernel * 1e-3) / 1e12
    kbase = f"build_refined_split_kernel<{nsys}>" if (33 <= nsys <= 40 and R == 1) else f"build_refined_reg_kernel<{nsys},{R}>"
    kname = kbase + (" (learned seed)" if learned_on else "")
    tps = KERNEL_TRAFFIC_PER_STENCIL.get(headline)
    # the FP64 work the refined kernel itself does: its FP64 residuals (n^2 R FMAs each, counted
    # by the build), at the FP64 FMA rate measured in this run
    res_fma = float(st_h.n_residuals) * nsys * nsys * R
    roof = {"kernel": kname, "bound": "fp64 pipe", "achieved": ach, "peak": fp64_peak.value, "unit": "TFLOP/s",
            "frac": ach / fp64_peak.value, "traffic": tps * n if tps else None,
            "flops": f"reference FP64 algorithm count per stencil ({flops_stencil:.0f}: n^3/3 + 2n^2R + assembly)",
            "peak_source": "FP64 FMA loop measured in this run (rbf_diag_fma_peak)",
            "traffic_source": "ncu dram__bytes_read+write of the same kernel on a 1M-point case, scaled by stencils"
                              if tps else "not captured",
            "note": "frac: the reference's FP64 algorithm (its FLOP count) at the measured FP64 peak, i.e. the "
                    "speed of light of a plain FP64 build; above 1 because this kernel factorises on the FP32 pipe "
                    "and spends its FP64 pipe on the residuals (fp64_residual_work below); the kernel itself is "
                    "bound by instruction issue and latency, not by one pipe",
            "fp64_residual_work": {"fma_per_s": res_fma / (ms_kernel * 1e-3),
                                   "frac_of_fp64_fma_rate": res_fma / (ms_kernel * 1e-3) / (fp64_peak.value * 0.5e12),
                                   "count": "FP64 residuals counted by the build x n^2 R FMAs"}}

    # ---- the adjoint of the build: gradients of <dW, W> with respect to the points (the
    # pullback of _build_weights), for a random cotangent of the headline operator
    adjoint = None
    if all(c in (0, 1, 3) for c, _ in cfg["ops"]):
        adj_b = pkg.find_neighbors(Xd, k=k, ctx=ctx)
        rp = build(headline, Xd, adj_b, sell=False)[0].row_ptr
        gen = torch.Generator(device=dev).manual_seed(7)
        dW = torch.rand((len(cfg["ops"]), n * k), generator=gen, device=dev, dtype=torch.float64) - 0.5
        ms_adj = timed(lambda: pkg.build_weights_backward(cfg["ops"], Xd, None, adj_b, basis, rp, dW, ctx=ctx),
                       2, 1)
        ms_adj_r = timed(lambda: pkg.build_weights_backward(cfg["ops"], Xd, None, adj_b, basis, rp, dW, ctx=ctx,
                                                            precision="fp32_refined"), 2, 1)
        g64 = sum(pkg.build_weights_backward(cfg["ops"], Xd, None, adj_b, basis, rp, dW, ctx=ctx))
        g32 = sum(pkg.build_weights_backward(cfg["ops"], Xd, None, adj_b, basis, rp, dW, ctx=ctx,
                                             precision="fp32_refined"))
        adjoint = {"ms": ms_adj, "stencils_per_s": n / (ms_adj * 1e-3), "ms_fp32_refined": ms_adj_r,
                   "refined_max_rel_diff_vs_fp64": float((g32 - g64).abs().max() / g64.abs().max()),
                   "ms_fp64_build": ms_b_64,
                   "kernel": "build_backward_kernel (FP64, one warp per stencil: assembly, LU with the weights' and "
                             "the adjoint's right-hand sides, pair gradients, atomic scatter); refined: "
                             "build_backward_refined_kernel (FP32 factor refined in FP64, FP64 fallback)"}
        if world == 1 and not args.no_cpu_baseline:
            # the reference's pullback restated in C (global coordinates, rook Bunch-Kaufman,
            # OpenMP on all host cores) on a sample of the same stencils
            from oracle import oracle as O
            m = 100_000
            a_h = adj_b[:m].cpu().numpy()
            dW_h = np.random.default_rng(8).random((len(cfg["ops"]), m, k)) - 0.5
            t0 = time.perf_counter()
            O.build_backward_c(X_h, X_h[:m], a_h, cfg["dim"], cfg["phs"], cfg["deg"], cfg["ops"], dW_h)
            t1 = time.perf_counter()
            adjoint["cpu"] = {"stencils_per_s": m / (t1 - t0), "cores": O.num_threads(), "kind": "port",
                              "sample": f"{m} stencils of the same cloud: the C restatement of the reference's "
                                        "pullback (global coordinates, rook Bunch-Kaufman)"}
        del dW, rp, adj_b, g64, g32

    # ---- the same workload after reorder_points (Morton order, the reference's locality
    # utility applied once): the apply's gathers become local
    perm, Xo = pkg.reorder_points(Xd, k, ctx=ctx)
    fo = fd[perm.long()].contiguous()
    adj_o = pkg.find_neighbors(Xo, k=k, ctx=ctx)
    Wo = build(headline, Xo, adj_o)[-1]
    ms_spmv_o = kernel_ms(lambda: Wo.apply(fo))
    gbs_o = apply_bytes / (ms_spmv_o * 1e-3) / 1e9
    Wo_sell, Wo.sell = Wo.sell, None
    ms_spmv_o_csr = kernel_ms(lambda: Wo.apply(fo))
    Wo.sell = Wo_sell
    gbs_o_csr = csr_bytes / (ms_spmv_o_csr * 1e-3) / 1e9
    ms_step_o = timed(lambda: step(headline, Xo, fo), max(1, args.steps // 2), 1)
    ms_reorder = timed(lambda: pkg.reorder_points(Xd, k, ctx=ctx), 3, 1)
    reordered = {"ms_reorder_points": ms_reorder, "ms_per_step": ms_step_o,
                 "stencils_per_s": n * world / (ms_step_o * 1e-3),
                 "apply": {"value": gbs_o, "unit": "GB/s", "ms": ms_spmv_o, "frac_of_hbm": gbs_o / hbm_peak,
                           "kernel": "spmv_sell_kernel (sliced-ELL copy)"},
                 "apply_csr": {"value": gbs_o_csr, "unit": "GB/s", "ms": ms_spmv_o_csr,
                               "frac_of_hbm": gbs_o_csr / hbm_peak, "kernel": "spmv_pair_kernel (CSR)"}}
    del Wo, Wo_sell, adj_o, Xo, fo

    # ---- e2e through the public API: host points in, host Laplacian of a host field out
    X_pin = torch.from_numpy(X_h).pin_memory()
    f_pin = torch.from_numpy(f_h).pin_memory()
    y_pin = torch.empty(n, dtype=torch.float64).pin_memory()

    def e2e_step():
        Xg = X_pin.to(dev, non_blocking=True)
        adj = pkg.find_neighbors(Xg, k=k, ctx=ctx)
        Ws = build(headline, Xg, adj)
        yy = Ws[-1].apply(f_pin.to(dev, non_blocking=True))
        y_pin.copy_(yy, non_blocking=True)

    ms_e2e = timed(e2e_step, max(1, args.steps // 2), 1)
    e2e = {"value": n * world / (ms_e2e * 1e-3), "unit": "stencils/s", "h2d_bytes_per_step": n * cfg["dim"] * 8 + n * 8,
           "d2h_bytes_per_step": n * 8}

    interp = None
    if rank == 0 and args.interp_n > 0:
        interp = interp_bench(pkg, torch, stream, args.interp_n, world == 1 and not args.no_cpu_baseline)

    cpu = None
    if cb is not None:
        cpu = {"value": cb["stencils_per_s"], "unit": "stencils/s", "cores": cb["cores"], "kind": "port",
               "sample": f"the first {cb['sample']} stencils of the same cloud: grid kNN over all {n} points + "
                         "raw-coordinate rook-BK build (rate extrapolated to the full cloud)"}

    if rank == 0:
        res = lambda s: float(s.n_residuals) / max(1, int(s.n_stencils))
        line = {
            "metric": METRIC, "value": value, "unit": "stencils/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("bf16 surrogate seed + " if learned_on else "") + "f32 factor + f64 refinement",
            "data": "synthetic (seeded)",
            "config": {"workload": cfg["desc"], "n": n, "k": k, "headline": headline,
                       "step": "kNN + " + ("features + MLP + " if learned_on else "")
                               + "build (CSR + sliced-ELL copy) + one apply (sliced)",
                       "l2": "inputs larger than L2 (CSR 12 B/nnz x nnz, adjacency 4 B x N x k)",
                       "parallelism": f"replicas x{world}"},
            "plain_fp64": {"value": n * world / (ms_fp64 * 1e-3), "unit": "stencils/s", "ms_per_step": ms_fp64},
            "fp32_refined_unseeded": {"value": n * world / (ms_fp32r * 1e-3), "unit": "stencils/s",
                                      "ms_per_step": ms_fp32r},
            "speedup_vs_plain_fp64": ms_fp64 / ms,
            "build_only": {"headline_ms": ms_b_h, "fp32_refined_ms": ms_b_32, "fp64_ms": ms_b_64,
                           "speedup_headline_vs_fp64": ms_b_64 / ms_b_h,
                           "headline_stencils_per_s": n / (ms_b_h * 1e-3),
                           "fp64_stencils_per_s": n / (ms_b_64 * 1e-3),
                           "kernel_ms": {"headline": ms_kernel, "fp32_refined": float(st32.ms_build),
                                         "fp64": float(st64.ms_build)}},
            "equal_error": {"vs_oracle": vs_oracle, "bar": 1e-8,
                            "vs_gpu_fp64_all_stencils": {"max_row_rel_weight_diff": err, "rms_rel_weight_diff": rms,
                                                         "operator_on_test_function_rel_diff": op_err,
                                                         "fp32_refined_unseeded_max_diff": err32},
                            "fallback_stencils": int(st_h.n_fallback)},
            "refinement": {"residuals_per_stencil": res(st_h), "unseeded_residuals_per_stencil": res(st32),
                           "fallback_unseeded": int(st32.n_fallback),
                           "seed_rel_err_mean_judged_by_solve": float(st_h.seed_rel_err_mean) if learned_on else None},
            "surrogate": training, "mlp": mlp,
            "apply": {"value": ord_gbs, "unit": "GB/s", "ms": ms_spmv_ord, "nnz": nnz,
                      "frac_of_hbm": ord_gbs / hbm_peak, "peak_source": hbm_src,
                      "kernel": "gather_perm_kernel + spmv_sell_perm_kernel (sliced copy in the points' Morton "
                                "order, x and y in the caller's order; the gather of x is counted in the time)",
                      "bytes": "sell_nnz*12 + (ne/32+1)*8 + 2*n*8 per apply (algorithmic); ms = kernel time "
                               "(library CUDA events)",
                      "ordered_copy_ms_once": ms_to_ordered, "equals_plain_sliced_bitwise": ord_equal,
                      "sliced_caller_layout": {"value": apply_gbs, "unit": "GB/s", "ms": ms_spmv,
                                               "ms_per_call_api": ms_spmv_api, "frac_of_hbm": apply_gbs / hbm_peak,
                                               "kernel": "spmv_sell_kernel (sliced-ELL copy written by the build, "
                                                         "rows in the caller's order)"},
                      "csr": {"value": csr_gbs, "unit": "GB/s", "ms": ms_spmv_csr, "frac_of_hbm": csr_gbs / hbm_peak,
                              "kernel": "spmv_pair_kernel", "bytes": "nnz*12 + (ne+1)*8 + 2*n*8"}},
            "reordered": reordered,
            "adjoint": adjoint,
            "algebra": algebra,
            "interpolator": interp,
            "knn": {"kernel": "knn_fast_kernel (grid buckets, FP32 keys, exact FP64 re-sort)", "ms": ms_knn_kernel,
                    "queries_per_s": n / (ms_knn_kernel * 1e-3),
                    "bytes": "(ns + ne) dim 8 + ne k 4 (points read, neighbour lists written)",
                    "GB_s": knn_bytes / (ms_knn_kernel * 1e-3) / 1e9,
                    "frac_of_hbm": knn_bytes / (ms_knn_kernel * 1e-3) / 1e9 / hbm_peak,
                    "bound": "not HBM: candidate selection (distance keys and the sorted k+8 list) on the "
                             "SM pipes; the HBM fraction shows how far it is from the traffic bound"},
            "kernels_ms": {"knn": ms_knn_kernel, "knn_per_call_api": ms_knn, "build_headline": ms_kernel,
                           "build_fp64": float(st64.ms_build), "spmv": ms_spmv, "spmv_ordered": ms_spmv_ord},
            "peaks": {"fp64_tflops_measured": fp64_peak.value, "fp32_tflops_measured": fp32_peak.value,
                      "hbm_gbs": hbm_peak},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
