#!/usr/bin/env python
"""Benchmark of the exact-GP hot path: conjugate MLL + gradient evaluations per
second at n = 16384, d = 8, Matern-5/2 ARD (X ~ N(0, I_8), lengthscales
log-uniform in [0.3, 3], variance 1, noise 1e-2, y drawn from the prior plus
noise in float64), mixed-precision form against the plain FP64 form.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one conjugate_mll value + gradient (lengthscales, variance,
obs_stddev, constant mean) over the whole synthetic dataset.  The exact GP
does not shard, so N > 1 runs N independent replicas (one per rank, weak
scaling).  Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLL+grad evals/s at n=16k: mixed vs FP64 form on one GB300 @ rel err ≤1e-6"
WORKLOAD = ("exact GP conjugate_mll + gradient, Matern-5/2 ARD, n=16384, d=8, X~N(0,I8), "
            "lengthscales log-U[0.3,3], variance 1, noise 1e-2, y = prior sample + noise")
PEAK_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}
# dram__bytes_read.sum + dram__bytes_write.sum of one adjoint GEMM launch
# (tc_gemm_kernel<MODE_GRAD, float16 wide>) on this workload at full size,
# n = 16384: 3.68 GB read + 41.1 MB written, from a one-pass ncu capture
# summarised in profiles/tc_gemm_grad_dram_n16384.txt.  The algorithmic operand
# volume is 0.54 GB (the upper triangle of V in float16 hi/lo): tiles of one
# L2-resident group share panels, the groups re-read them.
ADJOINT_TRAFFIC_BYTES_N16384 = 3.68e9 + 41.1e6


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", choices=["c2", "c3", "c4", "c5"], default="c2",
                   help="c2: the headline MLL+grad line (default); c3: n=65536, d=16 RBF "
                        "precision stress; c4: 512 batched GPs; c5: SGPR collapsed ELBO, "
                        "n=1e6, m=1024")
    p.add_argument("--n", type=int, default=None)
    p.add_argument("--d", type=int, default=None)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--seed", type=int, default=0)
    return p.parse_args()


def c2_inputs(n, d, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, d))
    ls = np.exp(rng.uniform(np.log(0.3), np.log(3.0), d))
    eps = rng.standard_normal(n)
    return x, ls, eps


def c2_y_device(x, ls, eps, device):
    """y = chol(K + (1e-6 + 1e-2) I) eps in float64 on the GPU (data generation,
    through the library's own float64 Gram and Cholesky)."""
    import torch

    import gpjax_gb300 as gpx
    X = torch.as_tensor(x, device=device)
    kern = gpx.kernels.Matern52(lengthscale=ls, variance=1.0)
    K = kern.gram(X).to_dense()
    K.diagonal().add_(1e-6 + 1e-2)
    L, info = gpx.linalg.cholesky_dense(K)
    del K
    assert int(info.item()) == 0
    y = L @ torch.as_tensor(eps, device=device)
    del L
    torch.cuda.empty_cache()
    return y


def c2_y_host(x, ls, eps):
    import scipy.linalg as sla
    from oracle import gp_oracle as O
    S = O.gram(O.MATERN52, x, ls, 1.0) + (1e-6 + 1e-2) * np.eye(len(x))
    return sla.cholesky(S, lower=True) @ eps


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return PEAK_FALLBACK, "fallback"


# ---------------------------------------------------------------------------
# CPU leg: the float64 oracle (the reference's op sequence) on the host cores
# ---------------------------------------------------------------------------
def c2_config(n, d, world=1):
    """The workload description both arms print (identical dicts)."""
    return {"workload": WORKLOAD if (n, d) == (16384, 8) else
            WORKLOAD.replace("n=16384, d=8", f"n={n}, d={d}"),
            "n": n, "d": d, "kernel": "Matern52",
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "working set (3 x n^2 float32 = 3.2 GB) larger than L2; no flush"}


def cpu_eval_setup(n, d, seed):
    x, ls, eps = c2_inputs(n, d, seed)
    return x, ls, c2_y_host(x, ls, eps)


def cpu_eval(x, y, ls):
    """Seconds of one float64 MLL + gradient of the oracle port on the host: the
    reference's op sequence (slogdet / solve through an LU factorisation, the
    gradient as reverse-mode differentiation forms it), row-blocked, torch
    threads."""
    from oracle import gp_oracle as O
    t0 = time.perf_counter()
    O.conjugate_mll_grad_lu(O.MATERN52, x, y, ls, 1.0, 0.1, 0.0)
    return time.perf_counter() - t0


def cpu_baseline(n_full, d, seed):
    """One full-size evaluation (n = 16384: ~10-30 s of host work)."""
    import torch
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    x, ls, y = cpu_eval_setup(n_full, d, seed)
    t = cpu_eval(x, y, ls)
    return {"value": 1.0 / t, "unit": "evals/s", "cores": threads, "kind": "port",
            "sample": (f"one float64 MLL+grad of the oracle port at the full workload (n={n_full}, "
                       f"d={d}): Sigma assembly, one LU shared by slogdet and solve, Sigma^-1 "
                       f"from the LU factors, gradient contraction; {t:.2f} s on {threads} "
                       "host threads")}


def run_reference(args):
    """--impl reference: the reference's algorithm for this path (the float64
    oracle port; JAX cannot be installed here) on the host cores, each timed
    step one full-size MLL + gradient evaluation of the same workload.
    Warm-up steps run the same evaluation at n = min(n, 2048) (thread pools
    and allocator)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    nw = min(args.n, 2048)
    xw, lw, yw = cpu_eval_setup(nw, args.d, args.seed)
    for _ in range(args.warmup):
        cpu_eval(xw, yw, lw)
    x, ls, y = cpu_eval_setup(args.n, args.d, args.seed)
    tot = 0.0
    for _ in range(args.steps):
        tot += cpu_eval(x, y, ls)
    value = args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": c2_config(args.n, args.d),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": (f"each timed step: one float64 MLL+grad of the oracle port "
                                    f"at the full workload (n={args.n}, d={args.d}); warm-up "
                                    f"steps at n={nw}")},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Replicas: the multi-GPU path (one process per GPU, no data-path collective)
# ---------------------------------------------------------------------------
class Replicas:
    """Host side of an N-GPU run of independent replicas: reads RANK /
    WORLD_SIZE / LOCAL_RANK, joins the process group for N > 1, and provides the
    barrier and the max-over-ranks time; the whole-job value is N x steps over
    that time.  The backend is NCCL on GPUs (gloo in the CPU tests)."""

    def __init__(self, backend: str):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)

    def barrier(self, device=None):
        import torch
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()
        if device is not None and device.type == "cuda":
            torch.cuda.synchronize(device)

    def max(self, v: float, device) -> float:
        if self.world == 1:
            return v
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def value(self, steps: int, seconds: float) -> float:
        return self.world * steps / seconds

    def close(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------
def run_gpu(args):
    import torch

    import gpjax_gb300 as gpx
    from gpjax_gb300 import _lib

    reps = Replicas("nccl")
    world, rank, local = reps.world, reps.rank, reps.local
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.lib()
    n, d = args.n, args.d

    # CPU baseline first (rank 0 at N = 1), before any process pool or GPU work
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(n, d, args.seed)

    x, ls, eps = c2_inputs(n, d, args.seed)
    X = torch.as_tensor(x, device=dev)
    y = c2_y_device(x, ls, eps, dev)
    theta = torch.tensor(list(ls) + [1.0, 0.1, 0.0], dtype=torch.float64, device=dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    grad = torch.zeros(d + 3, dtype=torch.float64, device=dev)
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def make_ws(prec):
        return _lib.workspace(lib.gpk_conjugate_mll_workspace_bytes(n, d, prec), dev)

    def step(prec, ws):
        _lib.call("gpk_conjugate_mll", _lib.MATERN52, n, d, X.data_ptr(), d, y.data_ptr(),
                  theta.data_ptr(), d, 1e-6, prec, 1, out.data_ptr(), grad.data_ptr(),
                  info.data_ptr(), ws.data_ptr(), ws.numel(), stream.cuda_stream)

    def barrier():
        reps.barrier(dev)

    def max_over_ranks(v):
        return reps.max(v, dev)

    # ---- plain FP64 form (reference precision) ----
    fp64 = None
    mll64 = g64 = None
    if args.fp64_steps > 0:
        ws64 = make_ws(_lib.PREC_FP64)
        step(_lib.PREC_FP64, ws64)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.fp64_steps):
            step(_lib.PREC_FP64, ws64)
        e1.record(stream)
        barrier()
        t64 = max_over_ranks(e0.elapsed_time(e1) / 1000.0)
        mll64, g64 = float(out.item()), grad.cpu().numpy().copy()
        fp64 = {"evals_per_s": world * args.fp64_steps / t64,
                "ms_per_step": 1000.0 * t64 / args.fp64_steps, "steps": args.fp64_steps}
        del ws64
        torch.cuda.empty_cache()

    # ---- mixed form, device-resident inputs (value) ----
    ws = make_ws(_lib.PREC_MIXED)
    for _ in range(args.warmup):
        step(_lib.PREC_MIXED, ws)
    barrier()
    nph = 7
    ph = [[torch.cuda.Event(enable_timing=True) for _ in range(nph)] for _ in range(args.steps)]
    ev_arrays = [ctypes_void_array(nph) for _ in range(args.steps)]
    for s in range(args.steps):
        for k in range(nph):
            ph[s][k].record(stream)  # torch creates the CUDA event on first record
            ev_arrays[s][k] = ph[s][k].cuda_event
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = lib.gpk_launch_count()
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for s in range(args.steps):
            lib.gpk_set_profile_events(ev_arrays[s], nph)
            step(_lib.PREC_MIXED, ws)
        e1.record(stream)
        barrier()
    lib.gpk_set_profile_events(None, 0)
    launches = lib.gpk_launch_count() - launches0
    t_dev = max_over_ranks(e0.elapsed_time(e1) / 1000.0)
    mll_mixed, g_mixed = float(out.item()), grad.cpu().numpy().copy()
    # mixed form: Gram; recursive Cholesky that also forms L^-1 (the T^T
    # products overlapped on the library's low-priority stream); alpha solve +
    # refinement; the adjoint GEMM; the join back to the caller's stream; the
    # float64 finalisation
    phase_names = ["gram", "factor", "solve_refine", "adjoint", "join", "finalize"]
    phases = {nm: float(np.mean([ph[s][k].elapsed_time(ph[s][k + 1]) for s in range(args.steps)]))
              for k, nm in enumerate(phase_names)}

    # ---- e2e through the public API with host buffers ----
    Xh = torch.as_tensor(x).pin_memory()
    yh = y.cpu().pin_memory()
    kern = gpx.kernels.Matern52(lengthscale=ls, variance=1.0)
    post = gpx.gps.Prior(kernel=kern) * gpx.likelihoods.Gaussian(n, obs_stddev=0.1)
    for p in (kern.lengthscale, kern.variance, post.likelihood.obs_stddev):
        p.to(dev).requires_grad_(True)

    def e2e_step():
        Xd = Xh.to(dev, non_blocking=True)
        yd = yh.to(dev, non_blocking=True)
        data = gpx.Dataset(X=Xd, y=yd, device=dev)
        for p in (kern.lengthscale, kern.variance, post.likelihood.obs_stddev):
            p.value.grad = None
        val = gpx.objectives.conjugate_mll(post, data, precision="mixed")
        val.backward()
        res = torch.cat([val.detach().reshape(1), kern.lengthscale.value.grad,
                         kern.variance.value.grad.reshape(1),
                         post.likelihood.obs_stddev.value.grad.reshape(1)])
        return res.cpu()

    for _ in range(2):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = e2e_step()
    barrier()
    t_e2e = max_over_ranks(time.perf_counter() - t0)
    h2d = Xh.numel() * 8 + yh.numel() * 8
    d2h = r.numel() * 8

    if rank != 0:
        reps.close()
        return

    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("bf16_tflops", PEAK_FALLBACK["bf16_tflops"]))
    # the factor phase (the largest share of the step): Cholesky n^3/3 + inverse n^3/3
    flops_factor = 2.0 * n ** 3 / 3.0
    ach_factor = flops_factor / (phases["factor"] / 1000.0) / 1e12
    # the adjoint: W = V V^T over the lower triangle, n^3/3
    flops_adjoint = n ** 3 / 3.0
    ach_adj = flops_adjoint / (phases["adjoint"] / 1000.0) / 1e12
    rel_mll = abs(mll_mixed - mll64) / abs(mll64) if mll64 is not None else None
    rel_grad = (float(np.linalg.norm(g_mixed - g64) / np.linalg.norm(g64))
                if g64 is not None else None)
    grad_comp = ({"names": [f"lengthscale[{k}]" for k in range(d)] +
                  ["variance", "obs_stddev", "constant"],
                  "fp64": [float(v) for v in g64],
                  "rel_err": [float(abs(a - b) / max(abs(b), 1e-300))
                              for a, b in zip(g_mixed, g64)]}
                 if g64 is not None else None)
    value = reps.value(args.steps, t_dev)
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 Gram + tf32x3 factor + f16x3 adjoint + f64 refinement/accumulation",
        "data": "synthetic",
        "config": c2_config(n, d, world),
        "roofline": {"bound": "tensor",
                     "kernel": "factor phase: recursive Cholesky + inverse L^-1 (tc_gemm_kernel "
                               "STORE_SPLIT / ADD_F32 products, leaf_chol_inv_kernel leaves, "
                               "float16 operand conversions), timed with CUDA events on the "
                               "library's stream at the phase boundaries",
                     "achieved": ach_factor, "peak": peak, "unit": "TFLOP/s",
                     "frac": ach_factor / peak, "peak_kind": f"{peak_kind} bf16 dense",
                     "traffic": None, "algorithmic_flops_per_launch": flops_factor,
                     "share_of_step": phases["factor"] / (1000.0 * t_dev / args.steps)},
        "roofline_adjoint": {"bound": "tensor",
                             "kernel": "tc_gemm_kernel<MODE_GRAD, float16 wide> (W = L^-T L^-1 "
                                       "tiles contracted with dK/dtheta), timed with its float16 "
                                       "conversion of L^-T (the adjoint phase)",
                             "achieved": ach_adj, "peak": peak, "unit": "TFLOP/s",
                             "frac": ach_adj / peak, "peak_kind": f"{peak_kind} bf16 dense",
                             "traffic": ADJOINT_TRAFFIC_BYTES_N16384 if n == 16384 else None,
                             "algorithmic_flops_per_launch": flops_adjoint},
        "phases_ms": phases,
        "fp64_form": fp64,
        "speedup_vs_fp64": (value / fp64["evals_per_s"]) if fp64 else None,
        "rel_err_mll_vs_fp64": rel_mll, "rel_err_grad_vs_fp64": rel_grad,
        "grad_components": grad_comp,
        "mll": mll_mixed,
        "e2e": {"value": reps.value(args.steps, t_e2e), "unit": "evals/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "gpjax_gb300.objectives.conjugate_mll(...).backward() from pinned host X, y"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    reps.close()


def ctypes_void_array(k):
    import ctypes
    return (ctypes.c_void_p * k)()


def run_c3(args):
    """Precision stress (workload c3): exact GP at n = 65536, d = 16, RBF ARD,
    X ~ U[0,1]^16, lengthscales log-U[0.1, 1], variance 1, noise 1e-3, jitter
    1e-6, y = a float64 prior sample plus noise (drawn through the library's
    float64 Gram and Cholesky), 4096 test points from the same X distribution.
    Mixed form against the plain float64 form on the MLL, its gradient and the
    predictive variance."""
    import torch

    from gpjax_gb300 import _lib
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lib = _lib.lib()
    n, d, t = args.n or 65536, args.d or 16, 4096
    rng = np.random.default_rng(args.seed)
    x = rng.uniform(0.0, 1.0, (n, d))
    ls = np.exp(rng.uniform(np.log(0.1), np.log(1.0), d))
    xt = rng.uniform(0.0, 1.0, (t, d))
    eps = rng.standard_normal(n)
    noise = 1e-3
    X = torch.as_tensor(x, device=dev)
    XT = torch.as_tensor(xt, device=dev)
    theta = torch.tensor(list(ls) + [1.0, float(np.sqrt(noise)), 0.0], dtype=torch.float64,
                         device=dev)
    stream = torch.cuda.current_stream(dev)
    # y = chol(K + (jitter + noise) I) eps, float64 (data generation, untimed)
    t0 = time.perf_counter()
    S = torch.empty((n, n), dtype=torch.float64, device=dev)
    _lib.call("gpk_gram", _lib.RBF, n, d, X.data_ptr(), d, theta.data_ptr(), d, _lib.F64,
              S.data_ptr(), n, stream.cuda_stream)
    S.diagonal().add_(1e-6 + noise)
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("gpk_lower_cholesky", n, _lib.F64, S.data_ptr(), n, None, info.data_ptr(),
              stream.cuda_stream)
    L = S
    Y = torch.zeros(n, dtype=torch.float64, device=dev)
    E = torch.as_tensor(eps, device=dev)
    for r0 in range(0, n, 8192):  # row blocks of L (lower triangle, upper part zero)
        Y[r0:r0 + 8192] = L[r0:r0 + 8192, :r0 + 8192] @ E[:r0 + 8192]
    torch.cuda.synchronize(dev)
    assert int(info.item()) == 0
    del S, L
    torch.cuda.empty_cache()
    t_gen = time.perf_counter() - t0
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    grad = torch.zeros(d + 3, dtype=torch.float64, device=dev)

    def timed(call, steps, warm):
        for _ in range(warm):
            call()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            call()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / 1000.0 / steps

    def mll(prec, steps, warm):
        ws = _lib.workspace(lib.gpk_conjugate_mll_workspace_bytes(n, d, prec), dev)
        tm = timed(lambda: _lib.call("gpk_conjugate_mll", _lib.RBF, n, d, X.data_ptr(), d,
                                     Y.data_ptr(), theta.data_ptr(), d, 1e-6, prec, 1,
                                     out.data_ptr(), grad.data_ptr(), info.data_ptr(),
                                     ws.data_ptr(), ws.numel(), stream.cuda_stream), steps, warm)
        res = (float(out.item()), grad.cpu().numpy().copy(), int(info.item()), tm)
        del ws
        torch.cuda.empty_cache()
        return res

    def predict(prec):
        mean = torch.zeros(t, dtype=torch.float64, device=dev)
        var = torch.zeros(t, dtype=torch.float64, device=dev)
        ws = _lib.workspace(lib.gpk_predict_workspace_bytes(n, t, d, prec), dev)
        tp = timed(lambda: _lib.call("gpk_predict", _lib.RBF, n, t, d, X.data_ptr(), d,
                                     Y.data_ptr(), XT.data_ptr(), d, theta.data_ptr(), d, 1e-6,
                                     1e-6, prec, mean.data_ptr(), var.data_ptr(), None, 0,
                                     info.data_ptr(), ws.data_ptr(), ws.numel(),
                                     stream.cuda_stream), 1, 0)
        res = (mean.cpu().numpy(), var.cpu().numpy(), int(info.item()), tp)
        del ws
        torch.cuda.empty_cache()
        return res

    mm, gm, im, tm = mll(_lib.PREC_MIXED, max(1, min(args.steps, 3)), 1)
    pm_mean, pm_var, ipm, tpm = predict(_lib.PREC_MIXED)
    line = {"workload": "c3 precision stress: exact GP MLL + gradient + predictive variance, "
                        f"RBF ARD, n={n}, d={d}, X~U[0,1]^{d}, lengthscales log-U[0.1,1], "
                        f"noise 1e-3, y = float64 prior sample + noise, {t} test points",
            "metric": f"MLL+grad evals/s at n={n}", "unit": "evals/s", "n": n, "d": d,
            "data": "synthetic", "y_generation_s": t_gen,
            "mixed": {"evals_per_s": 1.0 / tm, "ms_per_step": 1000.0 * tm, "mll": mm,
                      "info": im, "predict_ms": 1000.0 * tpm, "predict_info": ipm}}
    if args.fp64_steps > 0:
        m64, g64, i64, t64 = mll(_lib.PREC_FP64, 1, 0)
        p64_mean, p64_var, ip64, tp64 = predict(_lib.PREC_FP64)
        line["fp64_form"] = {"evals_per_s": 1.0 / t64, "ms_per_step": 1000.0 * t64, "mll": m64,
                             "info": i64, "predict_ms": 1000.0 * tp64, "predict_info": ip64}
        line["speedup_vs_fp64"] = t64 / tm
        line["rel_err_mll_vs_fp64"] = abs(mm - m64) / abs(m64)
        line["rel_err_grad_vs_fp64"] = float(np.linalg.norm(gm - g64) / np.linalg.norm(g64))
        line["max_rel_err_grad_component"] = float(np.max(np.abs(gm - g64) /
                                                          np.maximum(np.abs(g64), 1e-300)))
        line["max_rel_err_pred_var_vs_fp64"] = float(np.max(np.abs(pm_var - p64_var) /
                                                            np.abs(p64_var)))
        line["max_abs_err_pred_mean_vs_fp64"] = float(np.max(np.abs(pm_mean - p64_mean)))
        line["pred_var_range_fp64"] = [float(p64_var.min()), float(p64_var.max())]
    print(json.dumps(line), flush=True)


def run_c5(args):
    """SGPR (workload c5): collapsed ELBO + gradient (theta and Z), n = 1e6,
    m = 1024, d = 8; X a mixture of 16 Gaussians (means U[-5,5]^8, sd 0.5),
    y = sum_j sin(x_j) + N(0, 0.1^2), Z a random subset of X, RBF ARD with
    lengthscales log-U[0.5, 2]; mixed form against the float64 form."""
    import torch

    from gpjax_gb300 import _lib
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lib = _lib.lib()
    n, d, m = args.n or 1_000_000, args.d or 8, 1024
    rng = np.random.default_rng(args.seed)
    means = rng.uniform(-5.0, 5.0, (16, d))
    x = means[rng.integers(0, 16, n)] + 0.5 * rng.standard_normal((n, d))
    y = np.sin(x).sum(axis=1) + 0.1 * rng.standard_normal(n)
    z = x[rng.choice(n, m, replace=False)]
    ls = np.exp(rng.uniform(np.log(0.5), np.log(2.0), d))
    X, Y, Z = (torch.as_tensor(a, device=dev) for a in (x, y, z))
    theta = torch.tensor(list(ls) + [1.0, 0.1, 0.0], dtype=torch.float64, device=dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    grad = torch.zeros(d + 3, dtype=torch.float64, device=dev)
    gz = torch.zeros((m, d), dtype=torch.float64, device=dev)
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def run(prec, steps, warm):
        ws = _lib.workspace(lib.gpk_collapsed_elbo_workspace_bytes(n, m, d, prec), dev)
        call = lambda: _lib.call("gpk_collapsed_elbo", _lib.RBF, n, m, d, X.data_ptr(), d,
                                 Y.data_ptr(), Z.data_ptr(), d, theta.data_ptr(), d, 1e-6,
                                 prec, 1, out.data_ptr(), grad.data_ptr(), gz.data_ptr(),
                                 info.data_ptr(), ws.data_ptr(), ws.numel(),
                                 stream.cuda_stream)
        for _ in range(warm):
            call()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            call()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        t = e0.elapsed_time(e1) / 1000.0 / steps
        res = (float(out.item()), grad.cpu().numpy().copy(), gz.cpu().numpy().copy(),
               int(info.item()), t)
        del ws
        torch.cuda.empty_cache()
        return res

    em, gm, zm, im, tm = run(_lib.PREC_MIXED, max(1, min(args.steps, 5)), 1)
    e64, g64, z64, i64, t64 = run(_lib.PREC_FP64, max(1, min(args.fp64_steps, 2)), 1)
    print(json.dumps({
        "workload": f"c5 SGPR collapsed ELBO + gradient (theta, Z), RBF ARD, n={n}, m={m}, "
                    f"d={d}, X a 16-component Gaussian mixture",
        "metric": f"ELBO+grad evals/s at n={n}, m={m}", "unit": "evals/s",
        "n": n, "m": m, "d": d,
        "mixed": {"evals_per_s": 1.0 / tm, "ms_per_step": 1000.0 * tm, "elbo": em, "info": im},
        "fp64_form": {"evals_per_s": 1.0 / t64, "ms_per_step": 1000.0 * t64, "elbo": e64,
                      "info": i64},
        "speedup_vs_fp64": t64 / tm,
        "rel_err_elbo_vs_fp64": abs(em - e64) / abs(e64),
        "rel_err_grad_vs_fp64": float(np.linalg.norm(gm - g64) / np.linalg.norm(g64)),
        "rel_err_grad_z_vs_fp64": float(np.linalg.norm(zm - z64) / np.linalg.norm(z64)),
        "data": "synthetic"}), flush=True)


def c4_instances(count, seed):
    """Batched GPs (workload c4): n_i ~ U{64..2048}, d_i ~ U{2..10}, X ~ U[-1,1]^d, RBF or
    Matern-3/2 with probability 1/2, ARD lengthscales log-U[0.1, 2], variance
    log-U[0.5, 2], noise log-U[1e-4, 1e-1]; y = a random-Fourier-feature prior
    sample (100 frequencies, cos and sin features) + N(0, 0.05^2)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n, d = int(rng.integers(64, 2049)), int(rng.integers(2, 11))
        kind = 0 if rng.random() < 0.5 else 1  # RBF, Matern-3/2
        x = rng.uniform(-1.0, 1.0, (n, d))
        ls = np.exp(rng.uniform(np.log(0.1), np.log(2.0), d))
        var = float(np.exp(rng.uniform(np.log(0.5), np.log(2.0))))
        noise = float(np.exp(rng.uniform(np.log(1e-4), np.log(1e-1))))
        z = rng.standard_normal((100, d))
        if kind == 1:  # Matern-3/2 spectral density: multivariate t with 3 degrees of freedom
            z = z / np.sqrt(rng.chisquare(3.0, (100, 1)) / 3.0)
        proj = (x / ls) @ z.T
        feats = np.concatenate([np.cos(proj), np.sin(proj)], axis=1) * np.sqrt(var / 100)
        y = feats @ rng.standard_normal(200) + 0.05 * rng.standard_normal(n)
        out.append((kind, x, y, np.concatenate([ls, [var, np.sqrt(noise), 0.0]])))
    return out


def run_c4(args):
    """512 independent GPs per step: MLL + gradient of every instance.  The
    persistent plan (one kernel launch per step: one CTA per SM pulls instances
    from a size-sorted queue; tile configuration per size from the plan's
    autotuner) is captured once into a CUDA graph and replayed.  The earlier
    multi-stream form (one kernel chain per instance) is timed beside it."""
    import ctypes

    import torch

    from gpjax_gb300 import _lib
    from gpjax_gb300.objectives import BatchPlan
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lib = _lib.lib()
    count = 512
    insts = c4_instances(count, args.seed)
    xs = [torch.as_tensor(i[1], device=dev) for i in insts]
    ys = [torch.as_tensor(i[2], device=dev) for i in insts]
    ths = [torch.as_tensor(i[3], device=dev) for i in insts]
    kinds = [i[0] for i in insts]
    nls = [x.shape[1] for x in xs]
    t_plan0 = time.perf_counter()
    plan = BatchPlan(kinds, xs, ys, ths, nls, jitter=1e-6, want_grad=True, autotune=True)
    t_plan = time.perf_counter() - t_plan0
    for _ in range(max(args.warmup, 1)):
        plan.execute()
    torch.cuda.synchronize(dev)
    graph, mode = None, "eager"
    try:
        graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(s):
            with torch.cuda.graph(graph, stream=s):
                plan.execute()
        torch.cuda.current_stream(dev).wait_stream(s)
        graph.replay()
        torch.cuda.synchronize(dev)
        mode = "cuda graph of one persistent launch"
    except Exception:  # capture unsupported here: time the eager calls
        graph = None
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        graph.replay() if graph is not None else plan.execute()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    t = e0.elapsed_time(e1) / 1000.0 / args.steps
    mll = plan.mll.cpu().numpy()
    info = plan.info.cpu().numpy()
    # accuracy against the library's float64 form on a sample of instances
    # (all sizes; that form is held to the float64 oracle at 1e-10 by the tests)
    sample = list(range(0, count, 16))
    errs = []
    out64 = torch.zeros(1, dtype=torch.float64, device=dev)
    info64 = torch.zeros(1, dtype=torch.int32, device=dev)
    for k in sample:
        nk, dk = xs[k].shape
        g64 = torch.zeros(dk + 3, dtype=torch.float64, device=dev)
        ws64 = _lib.workspace(lib.gpk_conjugate_mll_workspace_bytes(nk, dk, _lib.PREC_FP64), dev)
        _lib.call("gpk_conjugate_mll", kinds[k], nk, dk, xs[k].data_ptr(), dk, ys[k].data_ptr(),
                  ths[k].data_ptr(), dk, 1e-6, _lib.PREC_FP64, 0, out64.data_ptr(),
                  g64.data_ptr(), info64.data_ptr(), ws64.data_ptr(), ws64.numel(),
                  stream.cuda_stream)
        ref = float(out64.item())
        errs.append(abs(mll[k] - ref) / abs(ref))
    # the multi-stream form, for comparison
    i32, i64, ptr = ctypes.c_int * count, ctypes.c_int64 * count, ctypes.c_void_p * count
    n = i64(*[x.shape[0] for x in xs])
    d = i32(*[x.shape[1] for x in xs])
    mll_o = torch.zeros(count, dtype=torch.float64, device=dev)
    grads_o = [torch.zeros(x.shape[1] + 3, dtype=torch.float64, device=dev) for x in xs]
    info_o = torch.zeros(count, dtype=torch.int32, device=dev)
    ws_o = _lib.workspace(lib.gpk_conjugate_mll_batched_workspace_bytes(count, n, d), dev)
    host = dict(kind=i32(*kinds), x=ptr(*[x.data_ptr() for x in xs]),
                ldx=i64(*[x.shape[1] for x in xs]), y=ptr(*[y.data_ptr() for y in ys]),
                th=ptr(*[t_.data_ptr() for t_ in ths]), nls=i32(*nls),
                out=ptr(*[mll_o.data_ptr() + 8 * k for k in range(count)]),
                g=ptr(*[g.data_ptr() for g in grads_o]))

    def step_old():
        _lib.call("gpk_conjugate_mll_batched", count, host["kind"], n, d, host["x"], host["ldx"],
                  host["y"], host["th"], host["nls"], 1e-6, 1, host["out"], host["g"],
                  info_o.data_ptr(), ws_o.data_ptr(), ws_o.numel(), stream.cuda_stream)

    step_old()
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(2):
        step_old()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    t_old = e0.elapsed_time(e1) / 1000.0 / 2
    sum_n3 = float(sum(float(x.shape[0]) ** 3 for x in xs))
    print(json.dumps({
        "workload": "c4 batched: 512 exact GPs, n_i~U{64..2048}, d_i~U{2..10}, RBF / Matern-3/2, "
                    "MLL + gradient of all instances per step",
        "metric": "MLL+grad steps/s (512 GPs per step)", "unit": "steps/s", "value": 1.0 / t,
        "ms_per_step": 1000.0 * t, "launch": mode, "gpu_launches_per_step": 1,
        "sum_n3": sum_n3, "tflops_n3_convention": sum_n3 / t / 1e12,
        "plan_create_s_incl_autotune": t_plan,
        "configs": {str(nn): plan.config(nn) for nn in (128, 512, 1024, 2048)},
        "dtype": "f32 products, f64 pivots, float-float refinement, f64 sums",
        "failed_instances": int((info != 0).sum()),
        "mll_rel_err_vs_fp64_form": {"instances": len(sample), "max": float(max(errs)),
                                  "median": float(np.median(errs))},
        "multi_stream_form": {"ms_per_step": 1000.0 * t_old, "steps_per_s": 1.0 / t_old},
        "data": "synthetic"}), flush=True)
    plan.close()


def main():
    args = parse_args()
    if args.impl == "reference":
        args.n, args.d = args.n or 16384, args.d or 8
        run_reference(args)
    elif args.workload == "c3":
        run_c3(args)
    elif args.workload == "c5":
        run_c5(args)
    elif args.workload == "c4":
        run_c4(args)
    else:
        args.n, args.d = args.n or 16384, args.d or 8
        run_gpu(args)


if __name__ == "__main__":
    main()
