#!/usr/bin/env python
"""Throughput of qLogNEI value + gradient at the headline point.

Workload: SingleTaskGP (Matern-5/2 ARD, d=20, n=4096 training points,
y = sum of Branin over 10 coordinate pairs + noise, lengthscales U[0.2, 1])
and qLogNoisyExpectedImprovement with 512 Sobol samples, evaluated with its
gradient on b=4096 t-batches of q=8 candidates per step (synthetic, seeded).
One step = one value+gradient call over the b t-batches with inputs resident
on the device; L2 is flushed (a 256 MB write) before every timed step.

Reports (one JSON line on rank 0):
  value      evaluations (t-batches) per second of the mixed-precision path
  e2e        the same through the public API with host buffers (H2D of X,
             D2H of value and gradient inside the timed region)
  roofline   the cross-covariance GEMMs (the dominant kernels), timed live
  cpu_baseline  the float64 CPU restatement of the reference path (oracle)
  plus the plain float64 GPU path's throughput and the mixed path's error
  against the float64 oracle.

``--impl reference`` times the reference's CPU float64 path (its restatement
under oracle/, since the reference's gpytorch/linear_operator dependencies
are not installed) on the host cores, on bounded samples of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import torch  # noqa: E402

METRIC = "qLogNEI value+grad evals/sec at n=4096,d=20,q=8 vs plain FP64 GPU @≤1e-5 rel err"
N_TRAIN, DIM, Q, S, B = 4096, 20, 8, 512, 4096
WORKLOAD = f"qlognei_branin_d{DIM}_n{N_TRAIN}_q{Q}_S{S}_b{B}"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--b", type=int, default=B)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--profile", action="store_true",
                   help="only warm up and run --steps mixed-precision steps between "
                        "cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    p.add_argument("--simt", action="store_true", help="FFMA GEMMs instead of tcgen05")
    p.add_argument("--profile-raw", action="store_true",
                   help="with --config optimize --profile: one raw-sample chunk instead of one round")
    p.add_argument("--profile-precision", default="mixed", choices=["mixed", "fp64"],
                   help="the path --profile runs (fp64: the plain float64 kernels)")
    p.add_argument("--config", default="headline",
                   choices=["headline", "many_gps", "optimize", "log_areas", "fit"],
                   help="many_gps: 64 GPs of uneven size in one tuned CUDA-graph launch; "
                        "optimize: one full acquisition optimisation step (d=50, 65536 raw "
                        "q-batches -> 64 restarts x q=16 -> L-BFGS-B); each prints its own line")
    p.add_argument("--maxiter", type=int, default=100, help="L-BFGS-B iterations (optimize)")
    p.add_argument("--streams", type=int, default=8, help="streams of the many-GP graph")
    p.add_argument("--profile-fit", action="store_true",
                   help="only build the model (training-side fit and operands) between "
                        "cudaProfilerStart/Stop, then exit")
    return p.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int) -> None:
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        rows = []
        if self.path.exists():
            for line in self.path.read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------- workload
def make_model(device, w):
    from botorch_gb300 import (ConstantMean, GaussianLikelihood, MaternKernel, ScaleKernel,
                               SingleTaskGP)

    covar = ScaleKernel(MaternKernel(nu=2.5, ard_num_dims=w.train_X.shape[-1], lengthscale=w.lengthscale),
                        outputscale=w.outputscale)
    return SingleTaskGP(w.train_X, w.train_Y, likelihood=GaussianLikelihood(w.noise), covar_module=covar,
                        mean_module=ConstantMean(w.mean_constant), device=device)


def make_acqf(model, w, precision):
    from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement

    torch.manual_seed(0)
    return qLogNoisyExpectedImprovement(model, w.train_X, sampler=SobolQMCNormalSampler(
        torch.Size([w.n_samples]), seed=w.seed), precision=precision)


def gemm_flops(rows: int, n: int, r: int) -> float:
    """Algorithmic flops of the two triangular cross-covariance GEMMs of one call.

    Forward V = K(X,Xt) L^-T: rows * n(n+1)/2 multiply-adds, plus the alpha
    column (rows * n) and P = V Vb^T (rows * n * r); adjoint D = H L^-1: rows *
    n(n+1)/2. Two flops per multiply-add.
    """
    tri = rows * n * (n + 1) / 2
    return 2.0 * (2 * tri + rows * n + rows * n * r)


def traffic_from_profiles() -> float | None:
    """DRAM bytes per GEMM launch at the bench workload, from the committed ncu summary
    of the kernel form the library runs (the two-SM pair)."""
    f = ROOT / "profiles" / "crosscov_gemm_pair_b1024.md"
    if f.exists():
        for line in f.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch_b4096:"):
                try:
                    return float(line.split(":", 1)[1])
                except ValueError:
                    return None
    return None


def measured_peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        return json.loads(f.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def time_steps(fn, steps: int, device, flush) -> list[float]:
    """Per-step device time (ms) with CUDA events on the launching stream; L2 flushed before each."""
    stream = torch.cuda.current_stream(device)
    times = []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        times.append((e0, e1))
    torch.cuda.synchronize(device)
    return [a.elapsed_time(b) for a, b in times]


def cpu_baseline(w, model_kw, n_batches: int = 32) -> dict:
    """The float64 oracle (restatement of the reference path) on the host cores."""
    from oracle.acquisition import QLogNoisyExpectedImprovement as OQLogNEI
    from oracle.gp import ExactGP

    om = ExactGP(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)
    torch.manual_seed(0)
    oa = OQLogNEI(om, w.train_X, w.n_samples, w.seed)
    Xs = w.X[:n_batches]
    oa.value_and_grad(Xs[:2])  # warm-up
    t0 = time.perf_counter()
    v, g = oa.value_and_grad(Xs)
    dt = time.perf_counter() - t0
    return {"value": n_batches / dt, "unit": "evals/s", "cores": torch.get_num_threads(), "kind": "port",
            "sample": f"{n_batches} t-batches of the headline workload, value+grad, float64, after init"}, (v, g)


# ---------------------------------------------------------------- our arm
def run_ours(args) -> None:
    from botorch_gb300 import _native as nat
    from botorch_gb300 import replicas
    from botorch_gb300 import testing as T

    world, rank, local = dist_info()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    b = args.b
    w = T.qlognei_branin(n=N_TRAIN, b=b, q=Q, d=DIM, seed=0)
    w.X = replicas.rank_candidates(w.X, rank)  # weak scaling: every rank its own candidates
    if args.profile_fit:
        from botorch_gb300.mll import exact_marginal_log_likelihood

        exact_marginal_log_likelihood(make_model(device, w))  # warm-up: library load, attributes
        torch.cuda.synchronize(device)
        torch.cuda.profiler.start()
        m = make_model(device, w)
        m.operands("mixed")
        exact_marginal_log_likelihood(m)
        torch.cuda.synchronize(device)
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_fit": True, "n": N_TRAIN, "jitter": m.train_jitter}))
        return
    model = make_model(device, w)
    acqf = make_acqf(model, w, args.profile_precision if args.profile else "mixed")
    acqf.check_status = False
    acqf.use_tensor_cores = not args.simt
    Xd = w.X.to(device).contiguous()
    out = (torch.empty(b, dtype=torch.float64, device=device),
           torch.empty(b, Q, DIM, dtype=torch.float64, device=device),
           torch.empty(b, dtype=torch.int32, device=device))
    eager_step = lambda: acqf.value_and_grad_raw(Xd, True, check=False, out=out)  # noqa: E731
    # the timed step: the whole call replayed from a CUDA graph (captured on the first call)
    step = lambda: acqf.graphed_value_and_grad(Xd, True, check=False)  # noqa: E731
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    for _ in range(max(args.warmup, 3)):
        eager_step()
        step()
    torch.cuda.synchronize(device)
    if args.profile:
        torch.cuda.profiler.start()
        for _ in range(args.steps):
            flush.zero_()
            eager_step()
        torch.cuda.synchronize(device)
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_steps": args.steps, "b": b, "status_ok": int(out[2].max().item()) == 0}))
        return
    lib = nat.lib()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    def load_for(seconds: float) -> None:  # the same step, untimed, to hold the clocks under load
        t_end = time.perf_counter() + seconds
        while time.perf_counter() < t_end:
            step()
            torch.cuda.synchronize(device)

    # the sampler window: 0.6 s of load, the timed steps, 0.3 s of load (the timed
    # region alone is shorter than the sampling period)
    with ClockSampler(local) as clk:
        load_for(0.6)
        t_wall0 = time.perf_counter()
        step_ms = time_steps(step, args.steps, device, flush)
        t_wall = time.perf_counter() - t_wall0
        load_for(0.3)
    # graph replays bypass the host-side counter: each replay runs the launches
    # recorded when the call was captured
    launches = acqf.graph_launches(b, Q) * args.steps
    torch.cuda.synchronize(device)
    launches0 = lib.bgb_launch_count()
    eager_ms = time_steps(eager_step, max(3, min(args.steps, 5)), device, flush)
    eager_launches_per_step = (lib.bgb_launch_count() - launches0) / len(eager_ms)
    total_ms = replicas.max_over_ranks(sum(step_ms), device)
    if world > 1:
        torch.distributed.barrier()
    graph_status = acqf._graphs[(b, Q, True, bool(acqf.use_tensor_cores), 0)]["out"][2]
    status_ok = int(out[2].max().item()) == 0 and int(graph_status.max().item()) == 0
    value = replicas.evals_per_second(world, b, args.steps, total_ms)
    eager_value = replicas.evals_per_second(1, b, len(eager_ms), sum(eager_ms))

    # roofline of the cross-covariance GEMMs, timed live per stage
    import ctypes
    stage = (ctypes.c_float * 7)()
    acq = acqf._acq_struct(Q)
    wp, wb = acqf._ws.get(lib.bgb_acq_workspace_bytes(ctypes.byref(acq), b))
    stage_runs = []
    for _ in range(3):
        flush.zero_()
        rc = lib.bgb_acq_forward_backward_timed(ctypes.byref(acq), Xd.data_ptr(), b, out[0].data_ptr(),
                                                out[1].data_ptr(), out[2].data_ptr(), wp, wb, stage,
                                                nat.stream_handle(device))
        nat.check(rc, "timed call")
        stage_runs.append(list(stage))
    st = [statistics.median(s[i] for s in stage_runs) for i in range(7)]
    names = ["kernel_build", "crosscov_gemm_fwd", "sigma_reduce", "batch_step", "mix_rows",
             "crosscov_gemm_adj", "adjoint"]
    peaks = measured_peaks()
    gemm_ms = st[1] + st[5]
    flops = gemm_flops(b * Q, N_TRAIN, acqf.r)
    achieved = flops / (gemm_ms / 1e3) / 1e12 / 2  # per launch: two launches per call
    per_launch_ms = gemm_ms / 2
    ach_tflops = (flops / 2) / (per_launch_ms / 1e3) / 1e12
    traffic = traffic_from_profiles()
    roofline = {"bound": "tensor", "kernel": "crosscov GEMM (triangular, fwd + adjoint)",
                "achieved": round(ach_tflops, 3), "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                "frac": round(ach_tflops / peaks.get("bf16_tflops", 1900.0), 5),
                "traffic": traffic, "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)",
                "algorithmic_tflop_per_launch": round(flops / 2 / 1e12, 4),
                "avg_launch_ms": round(per_launch_ms, 4)}
    del achieved

    # end to end through the public API: pinned host X -> value + grad back into
    # pinned host buffers, every step
    Xh = w.X.clone().pin_memory()
    vh = torch.empty(b, dtype=torch.float64).pin_memory()
    gh = torch.empty(b, Q, DIM, dtype=torch.float64).pin_memory()

    acqf.use_cuda_graphs = True

    def e2e_step():
        X = Xh.to(device, non_blocking=True).requires_grad_(True)
        v = acqf(X)
        (gx,) = torch.autograd.grad(v.sum(), X)
        vh.copy_(v.detach(), non_blocking=True)
        gh.copy_(gx, non_blocking=True)
        torch.cuda.current_stream(device).synchronize()

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize(device)
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize(device)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": round(world * b / e2e_s, 1), "unit": "evals/s", "h2d_bytes_per_step": int(Xh.numel() * 8),
           "d2h_bytes_per_step": int(vh.numel() * 8 + gh.numel() * 8)}
    if world > 1:
        torch.distributed.barrier()
    if rank != 0:
        torch.distributed.destroy_process_group()
        return

    # plain float64 GPU path (the denominator of the headline target): the same
    # b t-batches per call, replayed from a CUDA graph like the mixed path
    acq64 = make_acqf(model, w, "fp64")
    acq64.check_status = False
    step64 = lambda: acq64.graphed_value_and_grad(Xd, True, check=False)  # noqa: E731
    step64()  # capture
    ms64 = statistics.median(time_steps(step64, 2, device, flush))
    fp64_evals = b / (ms64 / 1e3)
    o64 = step64()
    torch.cuda.synchronize(device)

    # accuracy of the mixed path against the float64 oracle (and of the fp64 path)
    cpu = None
    err = {}
    if not args.no_cpu_baseline:
        cpu, (ov, og) = cpu_baseline(w, None, n_batches=32)
        nb = ov.shape[0]
        vm, gm_ = out[0][:nb].cpu(), out[1][:nb].cpu()
        err = {"value_rel_err_mixed": float((vm - ov).norm() / ov.norm()),
               "grad_rel_err_mixed": float((gm_ - og).norm() / og.norm()),
               "value_rel_err_fp64": float((o64[0][:nb].cpu() - ov).norm() / ov.norm()),
               "grad_rel_err_fp64": float((o64[1][:nb].cpu() - og).norm() / og.norm()),
               "error_sample": f"first {nb} t-batches vs float64 oracle, norm-wise"}

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16-split+f32+f64",
        "data": "synthetic (seeded Branin-sum GP workload)",
        "config": {"workload": WORKLOAD, "n": N_TRAIN, "d": DIM, "q": Q, "mc_samples": S,
                   "batch_per_call": b, "baseline_points_r": acqf.r, "kernel": "matern52",
                   "precision": "mixed: f32 kernel build, cross-covariance GEMMs on scaled f16 hi/lo "
                                "splits (3 tcgen05 products, f32 accumulation), f64 q x q "
                                "Cholesky + adjoint, f32 samples from exact f32 pairs of mu - best_f, "
                                "f64 accumulations", "l2": "flushed before each step (256 MB write)",
                   "parallelism": f"replicas, weak scaling over t-batches x{world}"},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
        "gpu_launches": int(launches), "launch_mode": "CUDA graph replay of the whole call",
        "launches_per_step": acqf.graph_launches(b, Q),
        "eager_evals_per_s": round(eager_value, 1),
        "eager_launches_per_step": eager_launches_per_step,
        "clocks": {**clk.summary(), "window": "0.6 s load, timed steps, 0.3 s load; 100 ms sampling"},
        "stage_ms": {k: round(v, 4) for k, v in zip(names, st)},
        "fp64_gpu_evals_per_s": round(fp64_evals, 1),
        "fp64_gpu_mode": f"CUDA graph replay, {b} t-batches per call (as the mixed path)",
        "speedup_vs_fp64_gpu": round(value / world / fp64_evals, 2),
        "status_ok": status_ok, "wall_s_timed": round(t_wall, 3), **err,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------- many GPs
MANY_METRIC = ("qLogNEI value+grad evals/sec, 64 GPs (n ~ logU[100,4000], d ~ U{4..30}), "
               "256 restarts x q=2, S=256, one CUDA-graph launch")


def run_many_gps(args) -> None:
    from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement
    from botorch_gb300 import testing as T
    from botorch_gb300.batched import Autotuner, ModelBatch, ModelGroup, apply_schedule

    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    works = T.many_gps(64, seed=0)
    t0 = time.perf_counter()
    acqfs, Xs = [], []
    for w in works:
        m = make_model(device, w)
        torch.manual_seed(0)
        acqfs.append(qLogNoisyExpectedImprovement(m, w.train_X, sampler=SobolQMCNormalSampler(
            torch.Size([w.n_samples]), seed=w.seed), precision="mixed"))
        Xs.append(w.X.to(device).contiguous())
    init_s = time.perf_counter() - t0
    evals = sum(x.shape[0] for x in Xs)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    def timed(fn, steps):
        times = []
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        return times

    # eager: one model after the other, library-default schedule
    for a in acqfs:
        apply_schedule(a, (True, 0))

    def eager():
        for a, x in zip(acqfs, Xs):
            a.value_and_grad_raw(x, True, check=False)

    for _ in range(max(args.warmup, 3)):
        eager()
    eager_ms = timed(eager, args.steps)
    tuner = Autotuner()
    mb = ModelBatch(acqfs, [tuple(x.shape) for x in Xs], n_streams=args.streams, tuner=tuner)
    for _ in range(max(args.warmup, 3)):
        mb.value_and_grad(Xs, check=False)
    graph_ms = timed(lambda: mb.value_and_grad(Xs, check=False), args.steps)
    status_ok = all(int(o[2].max().item()) == 0 for o in mb.out)
    # one launch per stage for all models (the default schedule: tensor-core GEMMs)
    for a in acqfs:
        apply_schedule(a, (True, 0))
    shapes = [tuple(x.shape) for x in Xs]
    group_ms, mg = None, None
    if ModelGroup.supported(acqfs, shapes):
        mg = ModelGroup(acqfs, shapes)
        for _ in range(max(args.warmup, 3)):
            mg.value_and_grad(Xs, check=False)
        if args.profile:  # one replay inside the profiler range, for a launch list
            torch.cuda.synchronize(device)
            torch.cuda.profiler.start()
            mg.value_and_grad(Xs, check=False)
            torch.cuda.synchronize(device)
            torch.cuda.profiler.stop()
            print(json.dumps({"profile_many_gps": True, "launches_per_step": mg.launches}))
            return
        group_ms = timed(lambda: mg.value_and_grad(Xs, check=False), args.steps)
        status_ok = status_ok and all(int(o[2].max().item()) == 0 for o in mg.out)
    choices = {}
    for key, sched in tuner.choice.items():
        label = f"{'tcgen05' if sched[0] else 'ffma'}/adj{sched[1] or 16}"
        choices[label] = choices.get(label, 0) + 1
    main_ms = group_ms if group_ms is not None else graph_ms
    launches = mg.launches if mg is not None else mb.launches
    line = {
        "metric": MANY_METRIC, "value": round(evals * args.steps / (sum(main_ms) / 1e3), 1),
        "unit": "evals/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(sum(main_ms) / len(main_ms), 4), "higher_is_better": True,
        "dtype": "f16-split+f32+f64", "data": "synthetic (seeded RFF GP draws)",
        "config": {"workload": "many_gps_64", "models": len(acqfs),
                   "n": sorted(int(a.model.n) for a in acqfs),
                   "restarts_per_model": 256, "q": 2, "mc_samples": 256,
                   "l2": "flushed before each step (256 MB write)", "streams": mb.n_streams},
        "form": "grouped plan: one launch per stage over all models" if mg is not None
                else "multi-stream CUDA graph of per-model launches",
        "eager_sequential_evals_per_s": round(evals * args.steps / (sum(eager_ms) / 1e3), 1),
        "multistream_graph_evals_per_s": round(evals * args.steps / (sum(graph_ms) / 1e3), 1),
        "multistream_graph_launches_per_step": int(mb.launches),
        "gpu_launches": int(launches * args.steps), "launches_per_step": int(launches),
        "schedule_buckets": len(tuner.choice), "schedule_choices": choices,
        "init_s": round(init_s, 2), "status_ok": status_ok,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- optimisation step
OPT_METRIC = ("qLogNEI acquisition optimisation step, d=50, n=4096, 65536 raw q-batches -> "
              "64 restarts x q=16, 1024 samples, L-BFGS-B")


def run_optimize(args) -> None:
    from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement
    from botorch_gb300 import testing as T
    from botorch_gb300.optim import (draw_sobol_samples, evaluate_raw, gen_candidates_scipy,
                                     initialize_q_batch)

    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    w = T.optimization_step()
    n, d = w.train_X.shape
    q, restarts, raw = w.extra["q"], w.extra["restarts"], w.extra["raw_samples"]
    t0 = time.perf_counter()
    model = make_model(device, w)
    acqfs = {}
    for precision in ("mixed", "fp64"):
        torch.manual_seed(0)
        acqfs[precision] = qLogNoisyExpectedImprovement(model, w.train_X, sampler=SobolQMCNormalSampler(
            torch.Size([w.n_samples]), seed=w.seed), precision=precision)
    acqf = acqfs["mixed"]
    torch.cuda.synchronize(device)
    init_s = time.perf_counter() - t0
    bounds = torch.stack([torch.zeros(d), torch.ones(d)]).double()
    # warm-up of the shapes and torch kernels used below (library set-up, graph
    # capture, the first use of torch's sampling kernels)
    bounds = bounds.to(device)  # raw samples drawn on the device
    Xr_w = draw_sobol_samples(bounds, 4096, q, seed=1)
    vr_w = evaluate_raw(acqf, Xr_w, 4096)
    initialize_q_batch(Xr_w.to(device), vr_w, restarts, eta=1.0,
                       generator=torch.Generator(device=device).manual_seed(1))
    Xw = torch.rand(restarts, q, d, dtype=torch.float64, device=device)
    acqf.graphed_value_and_grad(Xw, True)
    gen_candidates_scipy(Xw, acqf, 0.0, 1.0, {"maxiter": 2})
    torch.cuda.synchronize(device)
    t1 = time.perf_counter()
    X_raw = draw_sobol_samples(bounds, raw, q, seed=0)
    v_raw = evaluate_raw(acqf, X_raw, 4096)
    torch.cuda.synchronize(device)
    t2 = time.perf_counter()
    X0, _ = initialize_q_batch(X_raw.to(device), v_raw, restarts, eta=1.0,
                               generator=torch.Generator(device=device).manual_seed(0))
    if args.profile and args.profile_raw:  # the raw samples' draw and one forward-only chunk
        Xc = X_raw[:4096].to(device, torch.float64).contiguous()
        acqf.value_and_grad_raw(Xc, False, check=False)
        torch.cuda.synchronize(device)
        torch.cuda.profiler.start()
        draw_sobol_samples(bounds, raw, q, seed=0)
        acqf.value_and_grad_raw(Xc, False, check=False)
        torch.cuda.synchronize(device)
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_raw_draw": raw, "profile_raw_chunk": 4096}))
        return
    if args.profile:  # one round (evaluation + device L-BFGS-B step) inside the profiler range
        from botorch_gb300.lbfgsb import DeviceLbfgsb

        Xr = X0.reshape(restarts, q * d).contiguous().clone()
        lb = DeviceLbfgsb(Xr, torch.zeros(q * d), torch.ones(q * d), maxiter=args.maxiter)
        for r in range(args.warmup + 1):
            if r == args.warmup:
                torch.cuda.synchronize(device)
                torch.cuda.profiler.start()
            v, g = acqf.value_and_grad_raw(Xr.view(restarts, q, d), True, check=False)
            lb.step(v, g, sign=-1.0)
        torch.cuda.synchronize(device)
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_rounds": 1, "after_rounds": args.warmup, "summary": lb.summary.tolist()}))
        return
    # the default (the reference's): each restart its own L-BFGS-B, one batched
    # evaluation per round
    X, v = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": args.maxiter})
    torch.cuda.synchronize(device)
    t3 = time.perf_counter()
    info = gen_candidates_scipy.last_info
    v64, _ = acqfs["fp64"].value_and_grad_raw(X.contiguous(), False)
    err = float((v - v64).norm() / v64.norm())
    # the same per-restart mode with scipy's routine stepped per restart on the host
    t6 = time.perf_counter()
    Xs, vs = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": args.maxiter}, lbfgsb="scipy")
    torch.cuda.synchronize(device)
    t7 = time.perf_counter()
    info_s = gen_candidates_scipy.last_info
    # the reference's other mode on the same restarts: one L-BFGS-B on the sum
    t4 = time.perf_counter()
    _, va = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": args.maxiter}, use_parallel_mode=False)
    torch.cuda.synchronize(device)
    t5 = time.perf_counter()
    info_a = gen_candidates_scipy.last_info
    line = {
        "metric": OPT_METRIC, "value": round(t3 - t1, 4), "unit": "s", "n_gpus": 1,
        "higher_is_better": False, "dtype": "f16-split+f32+f64", "data": "synthetic (seeded RFF GP draw)",
        "config": {"workload": w.name, "n": n, "d": d, "q": q, "restarts": restarts,
                   "raw_samples": raw, "mc_samples": w.n_samples, "baseline_points_r": acqf.r,
                   "maxiter": args.maxiter},
        "raw_eval_s": round(t2 - t1, 4), "raw_evals_per_s": round(raw / (t2 - t1), 1),
        "lbfgsb_mode": info["mode"],
        "lbfgsb_s": round(t3 - t2, 4), "lbfgsb_iterations": info["nit"],
        "lbfgsb_iterations_per_restart_median": (sorted(info["nit_per_restart"])[len(info["nit_per_restart"]) // 2]
                                                 if "nit_per_restart" in info else None),
        "objective_evaluations": info["nfev"],
        "ms_per_objective_evaluation": round(1e3 * (t3 - t2) / max(info["nfev"], 1), 3),
        "evaluation_note": "per-restart mode: one evaluation = one round (all restarts that need f, g)",
        "restart_sum_start": -info["f0"], "restart_sum_final": -info["f"],
        "best_value": float(v.max()), "best_value_raw": float(v_raw.max()),
        "final_values_rel_err_vs_fp64": err, "init_s": round(init_s, 2),
        "launches_per_objective_evaluation": acqf.graph_launches(restarts, q),
        "lbfgsb_driver": info.get("driver"),
        "host_scipy_driver": {"lbfgsb_s": round(t7 - t6, 4), "iterations": info_s["nit"],
                              "rounds": info_s["nfev"],
                              "ms_per_round": round(1e3 * (t7 - t6) / max(info_s["nfev"], 1), 3),
                              "restart_sum_final": float(vs.sum()), "best_value": float(vs.max()),
                              "max_abs_candidate_diff_vs_device": float((Xs - X).abs().max())},
        "aggregated_mode": {"lbfgsb_s": round(t5 - t4, 4), "iterations": info_a["nit"],
                            "objective_evaluations": info_a["nfev"],
                            "ms_per_evaluation": round(1e3 * (t5 - t4) / max(info_a["nfev"], 1), 3),
                            "restart_sum_final": float(va.sum()), "best_value": float(va.max())},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- training side (fit step)
FIT_METRIC = ("exact-GP fit step (training covariance, psd_safe_cholesky, triangular inverse, alpha with "
              "refinement, exact MLL + gradient), steps/s at n=4096, d=20")
FP64_NOMINAL_TFLOPS = 1.25  # GB300 float64 (non-tensor), nominal


def run_fit(args) -> None:
    """One step of fit_gpytorch_mll's objective: refit the training cache at the current
    hyperparameters (bgb_gp_fit) and evaluate the MLL and its gradient (bgb_gp_mll)."""
    from botorch_gb300 import testing as T
    from botorch_gb300.mll import exact_marginal_log_likelihood

    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    w = T.qlognei_branin(n=N_TRAIN, b=1, q=1, d=DIM, seed=0)
    model = make_model(device, w)

    def refit():
        model.set_hyperparameters(noise=w.noise)  # a fresh training cache, as every fit step does

    def mll():
        exact_marginal_log_likelihood(model)

    for _ in range(max(args.warmup, 2)):
        refit()
        mll()
    torch.cuda.synchronize(device)
    steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(steps):
        refit()
    torch.cuda.synchronize(device)
    t_fit = (time.perf_counter() - t0) / steps
    t0 = time.perf_counter()
    for _ in range(steps):
        mll()
    torch.cuda.synchronize(device)
    t_mll = (time.perf_counter() - t0) / steps
    # the factorisation alone: K built on the device, blocked Cholesky in place
    import ctypes

    from botorch_gb300 import _native as nat

    lib = nat.lib()
    gp = model.gp_struct()
    Kd = torch.empty(N_TRAIN, N_TRAIN, dtype=torch.float64, device=device)
    Ad = torch.empty_like(Kd)
    cwb = lib.bgb_cholesky_workspace_bytes(N_TRAIN)
    cws = torch.empty(cwb, dtype=torch.uint8, device=device)
    Xt = model.train_inputs[0]
    info = ctypes.c_int32(0)
    stream = nat.stream_handle(device)
    chol_times = []
    for rep in range(4):
        nat.check(lib.bgb_kernel_matrix(ctypes.byref(gp), nat.ptr(Xt), N_TRAIN, nat.ptr(Xt), N_TRAIN,
                                        model.noise, nat.ptr(Kd), N_TRAIN, stream), "kernel matrix")
        Ad.copy_(Kd)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        nat.check(lib.bgb_cholesky(nat.ptr(Ad), N_TRAIN, N_TRAIN, ctypes.byref(info), nat.ptr(cws), cwb,
                                   stream), "cholesky")
        torch.cuda.synchronize(device)
        if rep > 0:
            chol_times.append(time.perf_counter() - t0)
    gpu_chol_ms = 1e3 * statistics.median(chol_times)
    del Kd, Ad, cws
    n = N_TRAIN
    # float64 flops (two per multiply-add): Cholesky n^3/3, triangular inverse n^3/3,
    # K^-1 = L^-T L^-1 (lower triangle) n^3/3
    flop_fit, flop_mll = 2 * n ** 3 / 3, n ** 3 / 3
    step_s = t_fit + t_mll
    achieved = (flop_fit + flop_mll) / step_s / 1e12
    # host reference: the same float64 factorisation and solves with all host threads
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    from oracle.gp import ExactGP
    from oracle.mll import exact_mll

    om = ExactGP(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)
    y = om.tf.transform(w.train_Y.double()).squeeze(-1)
    t0 = time.perf_counter()
    ExactGP(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)
    exact_mll(w.train_X, y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)
    cpu_s = time.perf_counter() - t0
    # the host LAPACK Cholesky alone of the same training covariance, all host threads
    from oracle.gp import kernel_matrix

    Kh = kernel_matrix(w.train_X, w.train_X, w.lengthscale, w.outputscale, w.kernel)
    Kh.diagonal().add_(w.noise)
    torch.linalg.cholesky(Kh)
    t0 = time.perf_counter()
    for _ in range(3):
        torch.linalg.cholesky(Kh)
    host_chol_ms = 1e3 * (time.perf_counter() - t0) / 3
    line = {"metric": FIT_METRIC, "value": round(1.0 / step_s, 3), "unit": "steps/s", "n_gpus": 1,
            "steps": steps, "warmup": max(args.warmup, 2), "ms_per_step": round(1e3 * step_s, 3),
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded Branin-sum GP workload)",
            "config": {"workload": "gp_fit_step_matern52_d20_n4096", "n": n, "d": DIM},
            "fit_ms": round(1e3 * t_fit, 3), "mll_grad_ms": round(1e3 * t_mll, 3),
            "cholesky_ms": round(gpu_chol_ms, 3), "host_lapack_cholesky_ms": round(host_chol_ms, 3),
            "roofline": {"bound": "fp64 pipe", "achieved": round(achieved, 4),
                         "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                         "frac": round(achieved / FP64_NOMINAL_TFLOPS, 4), "traffic": None,
                         "peak_source": "nominal GB300 float64 rate (not in MEASURED_PEAKS.json)"},
            "cpu_baseline": {"value": round(1.0 / cpu_s, 3), "unit": "steps/s", "cores": threads,
                             "kind": "port", "sample": "one fit step of the float64 oracle (torch, "
                                                       "LAPACK Cholesky + autograd MLL) at the same size"},
            "train_jitter": model.train_jitter}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- fused log-areas (qLogEHVI)
LA_METRIC = ("qLogEHVI fused log-areas forward+backward, (sample-batch, cell, subset) areas/s, "
             "m=2, q=4, 64 cells, 32768 sample-batches")


def _la_step_fns(w, go):
    """(step through the Jacobian route that FusedLogAreas takes under autograd,
    step through the reference extension's forward / backward contract)"""
    from botorch_gb300 import logei_fused as lf

    def step_jac():
        for obj, g in zip(w.obj_subsets, go):
            _, jac = lf.forward_with_jacobian(obj, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
            lf.backward_from_jacobian(g, jac)

    def step_recompute():
        for obj, g in zip(w.obj_subsets, go):
            lf.forward(obj, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
            lf.backward(g, obj, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
    return step_jac, step_recompute


def la_cpu_baseline(w, threads: int, sample_batches: int) -> tuple[float, str, str]:
    """Forward + backward of every subset size over the first `sample_batches` rows on
    `threads` host threads: the reference's own kernel (botorch/csrc/logei_fused.cpp)
    where it was compiled on this host (kind "reference"), else its bit-exact C
    restatement in the oracle (kind "port")."""
    from oracle import log_areas as ola
    from oracle.build import build_reference

    ref = build_reference()
    cpu = [o[:sample_batches].cpu() for o in w.obj_subsets]
    cl, cu = w.cell_lower.cpu(), w.cell_upper.cpu()
    gos = [torch.ones(sample_batches, w.nc, o.shape[1], dtype=o.dtype) for o in cpu]
    if ref is not None:
        torch.set_num_threads(threads)  # the reference kernel threads with at::parallel_for
        fwd = lambda o: ref.forward(o, cl, cu, w.tau_relu, w.tau_max)  # noqa: E731
        bwd = lambda g, o: ref.backward(g, o, cl, cu, w.tau_relu, w.tau_max)  # noqa: E731
        kind = "reference"
    else:
        fwd = lambda o: ola.forward(o, cl, cu, w.tau_relu, w.tau_max, threads=threads)  # noqa: E731
        bwd = lambda g, o: ola.backward(g, o, cl, cu, w.tau_relu, w.tau_max, threads=threads)  # noqa: E731
        kind = "port"
    fwd(cpu[0][:8])  # load / build
    t0 = time.perf_counter()
    for o, g in zip(cpu, gos):
        fwd(o)
        bwd(g, o)
    dt = time.perf_counter() - t0
    areas = sample_batches * w.nc * sum(int(o.shape[1]) for o in cpu)
    return areas / dt, f"{sample_batches} of {w.B} sample-batches, all subset sizes, fwd+bwd", kind


def run_log_areas(args) -> None:
    from botorch_gb300 import _native as nat
    from botorch_gb300 import logei_fused as lf
    from botorch_gb300.testing import log_areas_workload

    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    lib = nat.lib()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)
    res = {}
    for tag, dtype in (("f64", torch.float64), ("f32", torch.float32)):
        w = log_areas_workload(dtype=dtype, device=device)
        g = torch.Generator().manual_seed(1)
        go = [torch.randn(w.B, w.nc, o.shape[1], generator=g, dtype=torch.float64).to(device, dtype)
              for o in w.obj_subsets]
        step, step_rc = _la_step_fns(w, go)
        for _ in range(max(args.warmup, 3)):
            step()
            step_rc()
        torch.cuda.synchronize(device)
        n0 = lib.bgb_launch_count()
        with ClockSampler(0) as clk:
            ms = time_steps(step, args.steps, device, flush)
        launches = lib.bgb_launch_count() - n0
        ms_rc = time_steps(step_rc, args.steps, device, flush)
        # per-kernel times (forward and backward of the largest subset size, i = 2)
        obj2, go2 = w.obj_subsets[1], go[1]
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        flush.zero_()
        ev[0].record(stream)
        lf.forward(obj2, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
        ev[1].record(stream)
        lf.backward(go2, obj2, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
        ev[2].record(stream)
        _, jac2 = lf.forward_with_jacobian(obj2, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
        ev[3].record(stream)
        lf.backward_from_jacobian(go2, jac2)
        ev[4].record(stream)
        torch.cuda.synchronize(device)
        jac_bytes2 = jac2.numel() * jac2.element_size()
        del jac2
        # end to end: host objective samples in (pinned), areas and gradients out (pinned)
        h_obj = [o.cpu().pin_memory() for o in w.obj_subsets]
        h_go = [x.cpu().pin_memory() for x in go]
        h_out = [torch.empty(w.B, w.nc, o.shape[1], dtype=dtype).pin_memory() for o in w.obj_subsets]
        h_grad = [torch.empty(o.shape, dtype=dtype).pin_memory() for o in w.obj_subsets]

        def e2e_step():  # through the autograd function, as the acquisition function calls it
            for ho, hg, hout, hgr in zip(h_obj, h_go, h_out, h_grad):
                o = ho.to(device, non_blocking=True).requires_grad_(True)
                gg = hg.to(device, non_blocking=True)
                a = lf.FusedLogAreas.apply(o, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
                (gr,) = torch.autograd.grad(a, o, gg)
                hout.copy_(a.detach(), non_blocking=True)
                hgr.copy_(gr, non_blocking=True)
            torch.cuda.current_stream(device).synchronize()

        e2e_step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / args.steps
        h2d = sum(x.numel() * x.element_size() for x in h_obj + h_go)
        d2h = sum(x.numel() * x.element_size() for x in h_out + h_grad)
        mean_ms = sum(ms) / len(ms)
        # algorithmic bytes: objective samples and cells read once, areas written (forward);
        # grad_out read, gradient written (backward)
        bytes_step = sum(o.numel() * o.element_size() * 2 + x.numel() * x.element_size() * 2
                         + 2 * x.numel() * o.shape[2] * o.shape[3] * o.element_size()
                         for o, x in zip(w.obj_subsets, go))
        res[tag] = {"areas_per_s": w.areas_per_step() / (mean_ms / 1e3), "ms_per_step": mean_ms,
                    "recompute_areas_per_s": w.areas_per_step() / (sum(ms_rc) / len(ms_rc) / 1e3),
                    "fwd_ms_i2": ev[0].elapsed_time(ev[1]), "bwd_ms_i2": ev[1].elapsed_time(ev[2]),
                    "fwdjac_ms_i2": ev[2].elapsed_time(ev[3]), "bwdjac_ms_i2": ev[3].elapsed_time(ev[4]),
                    "jac_bytes_i2": jac_bytes2,
                    "e2e_areas_per_s": w.areas_per_step() / e2e_s, "h2d": h2d, "d2h": d2h,
                    "launches": launches, "clocks": clk.summary(), "bytes_step": bytes_step,
                    "log_fatplus_per_step": 2 * w.B * w.nc * w.m * sum(int(o.shape[1] * o.shape[2])
                                                                        for o in w.obj_subsets)}
        w_cpu = w
    peaks = measured_peaks()
    r = res["f64"]
    achieved_gbs = r["bytes_step"] / (r["ms_per_step"] / 1e3) / 1e9
    threads = os.cpu_count() or 1
    cpu_value, cpu_sample, cpu_kind = (None, None, None)
    if not args.no_cpu_baseline:
        w64 = log_areas_workload(dtype=torch.float64)
        cpu_value, cpu_sample, cpu_kind = la_cpu_baseline(w64, threads, 2048)
    line = {
        "metric": LA_METRIC, "value": round(r["areas_per_s"], 1), "unit": "areas/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(r["ms_per_step"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded objective samples, 63-point front)",
        "config": {"workload": "log_areas_m2_q4_nc64_B32768", "B": w_cpu.B, "q": 4, "m": 2, "cells": 64,
                   "areas_per_step": w_cpu.areas_per_step(), "l2": "flushed before each step (256 MB write)"},
        "e2e": {"value": round(r["e2e_areas_per_s"], 1), "unit": "areas/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"]},
        "roofline": {"bound": "fp64 pipe (transcendentals); hbm shown", "achieved": round(achieved_gbs, 1),
                     "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": round(achieved_gbs / peaks["hbm_gbs"], 4) if peaks.get("hbm_gbs") else None,
                     "traffic": None},
        "route": "Jacobian kept by the forward, backward = HBM contraction (FusedLogAreas under autograd)",
        "recompute_route_areas_per_s": round(r["recompute_areas_per_s"], 1),
        "kernel_ms_subset2": {"forward": round(r["fwd_ms_i2"], 4), "backward": round(r["bwd_ms_i2"], 4),
                              "forward_jacobian": round(r["fwdjac_ms_i2"], 4),
                              "backward_from_jacobian": round(r["bwdjac_ms_i2"], 4),
                              "jacobian_bytes": r["jac_bytes_i2"]},
        "f32": {"value": round(res["f32"]["areas_per_s"], 1), "ms_per_step": round(res["f32"]["ms_per_step"], 4),
                "recompute_route_areas_per_s": round(res["f32"]["recompute_areas_per_s"], 1),
                "e2e": round(res["f32"]["e2e_areas_per_s"], 1),
                "kernel_ms_subset2": {"forward": round(res["f32"]["fwd_ms_i2"], 4),
                                      "backward": round(res["f32"]["bwd_ms_i2"], 4),
                                      "forward_jacobian": round(res["f32"]["fwdjac_ms_i2"], 4),
                                      "backward_from_jacobian": round(res["f32"]["bwdjac_ms_i2"], 4)}},
        "cpu_baseline": None if cpu_value is None else {
            "value": round(cpu_value, 1), "unit": "areas/s", "cores": threads, "kind": cpu_kind,
            "sample": cpu_sample + (" (the reference's own kernel, compiled on this host)" if cpu_kind == "reference"
                                    else " (C restatement of the reference kernel, bit-exact to it on x86-64)")},
        "gpu_launches": int(r["launches"]), "clocks": r["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_log_areas_reference(args) -> None:
    """Reference arm of the log-areas benchmark on all host cores: the reference's own
    kernel (botorch/csrc/logei_fused.cpp) where it was compiled on this host, else its
    C restatement (bit-exact to it on x86-64)."""
    world, rank, _ = dist_info()
    if rank != 0:
        return
    from botorch_gb300.testing import log_areas_workload

    w = log_areas_workload(dtype=torch.float64)
    threads = os.cpu_count() or 1
    sample = 1024
    for _ in range(max(args.warmup, 1)):
        la_cpu_baseline(w, threads, 256)
    vals = [la_cpu_baseline(w, threads, sample) for _ in range(args.steps)]
    value = statistics.median(v for v, _, _ in vals)
    line = {"metric": LA_METRIC, "value": round(value, 1), "unit": "areas/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded objective samples, 63-point front)",
            "impl": "reference",
            "config": {"workload": "log_areas_m2_q4_nc64_B32768", "B": w.B, "q": 4, "m": 2, "cells": 64},
            "cpu_baseline": {"value": round(value, 1), "unit": "areas/s", "cores": threads,
                             "kind": vals[0][2], "sample": vals[0][1]},
            "e2e": {"value": round(value, 1), "unit": "areas/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- reference arm
def run_reference(args) -> None:
    world, rank, _ = dist_info()
    if rank != 0:
        return
    from botorch_gb300 import testing as T
    from oracle.acquisition import QLogNoisyExpectedImprovement as OQLogNEI
    from oracle.gp import ExactGP

    torch.set_num_threads(os.cpu_count() or 1)
    w = T.qlognei_branin(n=N_TRAIN, b=args.b, q=Q, d=DIM, seed=0)
    om = ExactGP(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)
    torch.manual_seed(0)
    oa = OQLogNEI(om, w.train_X, w.n_samples, w.seed)
    per_step = 8
    for i in range(max(args.warmup, 1)):
        oa.value_and_grad(w.X[i * per_step:(i + 1) * per_step])
    t0 = time.perf_counter()
    for i in range(args.steps):
        j = (i * per_step) % (args.b - per_step)
        oa.value_and_grad(w.X[j:j + per_step])
    dt = time.perf_counter() - t0
    value = per_step * args.steps / dt
    cores = torch.get_num_threads()
    line = {"metric": METRIC, "value": round(value, 3), "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Branin-sum GP workload)", "impl": "reference",
            "config": {"workload": WORKLOAD, "n": N_TRAIN, "d": DIM, "q": Q, "mc_samples": S,
                       "batch_per_call": per_step, "workload_batch": args.b,
                       "parallelism": "host CPU, rank 0"},
            "rate_basis": "per t-batch value+gradient evaluation; each step is a bounded sample of "
                          f"{per_step} of the workload's {args.b} t-batches",
            "cpu_baseline": {"value": round(value, 3), "unit": "evals/s", "cores": cores, "kind": "port",
                             "sample": f"{per_step} t-batches per step, value+grad, float64"},
            "e2e": {"value": round(value, 3), "unit": "evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference CPU float64 path via its restatement in oracle/ (gpytorch and "
                    "linear_operator, which hold the reference's arithmetic, are not installable offline)"}
    print(json.dumps(line), flush=True)


def main() -> None:
    args = parse()
    if args.impl == "reference" and args.config == "log_areas":
        run_log_areas_reference(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.config == "log_areas":
        run_log_areas(args)
    elif args.config == "many_gps":
        run_many_gps(args)
    elif args.config == "optimize":
        run_optimize(args)
    elif args.config == "fit":
        run_fit(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
