"""Benchmark: log-likelihood + exact gradient evaluations per second on the
non-stationary 200 x 200 x 24 advection-diffusion model (960,000 nodes), mixed
precision, one GPU; plus 256-column posterior sampling and the CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one evaluation of the objective and its gradient in all parameters
(assemble Q and Q_c, two factorisations, two selected inversions, the
conditional-mean solve with FP64 refinement, the adjoint), exactly the work of
the reference's logLike(par, grad=True) with exact instead of stochastic traces.
Under torchrun (N > 1) every rank runs an independent replica (the
factorisation does not shard without a Schur-complement exchange per tree
level), value = total evaluations / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

# The CPU legs run scipy / numpy on the host: pin the BLAS thread count before
# numpy loads (reported in the JSON line).
os.environ.setdefault("OPENBLAS_NUM_THREADS", str(os.cpu_count() or 1))

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "logL+grad evals/s & samples/s, 200x200x24 SPDE: mixed+learned vs FP64 plain"


# DRAM bytes per algorithmic flop of the tensor-core product, from the ncu
# capture of the largest cluster-pair launch at 100 x 100 x 24 (an inverse-block
# product of 4.430e11 flops: 1.285e9 bytes read, 0.157e9 written).
TC_DRAM_BYTES_PER_FLOP = 1.442e9 / 4.430e11


def _tf32_tflops(torch, n=8192, reps=10):
    """cuBLAS FP32 GEMM with TF32 tensor cores allowed, best of `reps` (the
    single-pass TF32 rate; a 3xTF32 product issues three such passes)."""
    try:
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = True
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        torch.matmul(a, b)
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        torch.backends.cuda.matmul.allow_tf32 = prev
        del a, b
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    except Exception:
        return None


def _dgemm_tflops(torch, n=4096, reps=5):
    """cuBLAS FP64 GEMM, best of `reps`: the ceiling of the FP64 plan's dense
    products (the plain FP64 path the mixed plan is compared with)."""
    try:
        a = torch.randn(n, n, device="cuda", dtype=torch.float64)
        b = torch.randn(n, n, device="cuda", dtype=torch.float64)
        torch.matmul(a, b)
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    except Exception:
        return None


def _blas_threads():
    return {"OPENBLAS_NUM_THREADS": os.environ.get("OPENBLAS_NUM_THREADS"), "host_cores": os.cpu_count()}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "of measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "of fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", "0", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(s[0]) for s in self.samples if len(s) >= 7 and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) >= 7 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 7 for i in range(4) if s[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _cpu_case(M=30, N=30, T=24):
    """The reference's CPU path (oracle restatement: SuperLU / LAPACK factor,
    Hutchinson traces with the reference's 100 probes) on an M x N x T sub-grid
    of the same model family; the full 960k-node grid is out of reach on the CPU."""
    from oracle.spde_oracle import OracleGrid, OracleModel
    from spdepy_gb300.workloads import fourier_velocity
    g = OracleGrid(np.arange(M, dtype=float), np.arange(N, dtype=float), np.arange(T, dtype=float), None, 5)
    we, wn = fourier_velocity(M, N, seed=1)
    ww = g.assimilate_adv(we, wn)
    mod = OracleModel(g, "cov-advection-var-diffusion", "ani", 3, ww=ww)
    rng = np.random.default_rng(1)
    nb2 = 25
    par = np.hstack([np.full(nb2, np.log(0.3)), np.full(nb2, np.log(0.5)), rng.normal(0, 0.3, nb2),
                     rng.normal(0, 0.3, nb2), 1.0, 0.0, np.log(0.3), np.log(0.5), np.sqrt(0.5), 0.0, np.log(100.0)])
    idx = np.sort(rng.choice(g.n, g.n // 100, replace=False))
    y = rng.normal(size=idx.size)
    return g.n, (lambda k: mod.loglike(par, y, idx, grad=True, nh1=100, seed=k))


# Sub-grids timed for the CPU figures (T = 24, as the benchmarked workload):
# the cpu_baseline of the GPU arm (about 20 s of CPU work) and the longer ladder
# of the reference arm (up to 60,000 nodes, about 3 minutes per pass).
CPU_LADDER = ((20, 20), (30, 30))
CPU_LADDER_REFERENCE = ((30, 30), (40, 40), (50, 50))


def _cpu_ladder(ladder=CPU_LADDER):
    return [_cpu_case(M, N) for M, N in ladder]


def _time_ladder(cases, seed):
    """One bounded sample: one reference-path evaluation per sub-grid; [(nodes, seconds)]."""
    out = []
    for n, evaluate in cases:
        t0 = time.perf_counter()
        evaluate(seed)
        out.append((n, time.perf_counter() - t0))
    return out


def _cpu_figures(points, n_full, passes):
    """Scale the sampled CPU cost to one evaluation of the n_full-node workload.

    `value` scales the largest sub-grid's seconds per evaluation linearly in the
    node count.  The sparse factorisation's cost grows faster than that (the
    fitted exponent is reported), so this overstates the CPU's rate on the full
    workload and understates the GPU's advantage.  The power-law extrapolation is
    reported beside it for information."""
    ns = np.array([p[0] for p in points], float)
    ts = np.array([p[1] for p in points], float)
    expo = float(np.polyfit(np.log(ns), np.log(ts), 1)[0]) if len(points) > 1 else 1.0
    n1, t1 = ns[-1], ts[-1]
    linear = 1.0 / (t1 * n_full / n1)
    power = 1.0 / (t1 * (n_full / n1) ** expo)
    ladder = ", ".join(f"{int(n)} nodes: {t:.2f} s" for n, t in zip(ns, ts))
    sample = (f"reference CPU path (SuperLU factor, Hutchinson gradient nh1=100) on sub-grids of the same model "
              f"at T=24, seconds per evaluation averaged over {passes} pass(es): {ladder}; scaled linearly in "
              f"nodes to the {n_full}-node workload (the fitted cost exponent is {expo:.2f}, so this overstates "
              f"the CPU rate)")
    return {"value": linear, "unit": "evals/s", "cores": os.cpu_count() or 1, "kind": "port", "sample": sample,
            "sample_evals_per_s": 1.0 / t1, "sample_nodes": int(n1), "cost_exponent": expo,
            "value_power_law": power, "blas_threads": _blas_threads()}


def cpu_baseline(n_full, passes=1):
    cases = _cpu_ladder()
    runs = [_time_ladder(cases, k) for k in range(passes)]
    points = [(runs[0][i][0], float(np.mean([r[i][1] for r in runs]))) for i in range(len(cases))]
    return _cpu_figures(points, n_full, passes)


def learned_pcg_leg(train_steps=5000, size=(400, 400, 48)):
    """Conditional-mean solve by PCG on the 400 x 400 x 48 non-stationary
    workload (7.68M nodes, seed 2, 1 % observed, right-hand side tau S^T y with
    synthetic y ~ N(0, 1)) with the learned preconditioner trained on
    `train_steps` systems at 100 x 100 x 12 drawn from the prior, against Jacobi,
    incomplete-Cholesky (IC(0), natural order, level-scheduled) and plain CG;
    tolerance 1e-6 relative residual (true residual reported)."""
    import torch
    from spdepy_gb300.precond import LearnedPreconditioner, system_maker
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion
    wt = nonstationary_advection_diffusion(M=100, N=100, T=12)
    mt = build_model(wt, "iterative")
    lp = LearnedPreconditioner(seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = lp.train(system_maker(wt, mt), steps=train_steps, probes=4, lr=3e-3, seed=1)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    we = nonstationary_advection_diffusion(M=size[0], N=size[1], T=size[2], seed=2)
    me = build_model(we, "iterative")
    me._assemble(we.par)
    rng = np.random.default_rng(2)
    n = we.grid.n
    idx = np.sort(rng.choice(n, n // 100, replace=False))
    me.plan.set_obs(idx)
    tau = float(np.exp(we.par[-1]))
    b = np.zeros(n)
    b[idx] = tau * rng.normal(size=idx.size)
    bt = torch.as_tensor(b).cuda()
    out = {"workload": f"nonstationary advection-diffusion {size[0]}x{size[1]}x{size[2]} ({n} nodes), seed 2, 1% observed",
           "tol": 1e-6,
           "training": {"systems": train_steps, "grid": "100x100x12", "probes_per_system": 4,
                        "seconds": round(t_train, 2), "loss_first10": float(np.mean(hist[:10])),
                        "loss_last100": float(np.mean(hist[-100:]))}}
    for kind in ("learned", "jacobi", "ic0", "none"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        wts = lp.weights(me.plan, True, tau) if kind == "learned" else None
        x, it, rel = me.plan.pcg(bt, True, tau, kind, w=wts, tol=1e-6, maxit=5000, check=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[kind] = {"iterations": it, "relres": rel, "ms": round(dt * 1e3, 2), "ms_per_iteration": round(dt * 1e3 / max(it, 1), 3)}
    # 64 posterior draws without a factorisation: x = mu + A^-1 (B^T e1 + sqrt(tau) S^T e2), Q = B^T B
    me.initFit(b[idx] / tau, idx=idx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xs, its = me.samplePosteriorPCG(n=64, precond=lp, seed=3, tol=1e-6)
    torch.cuda.synchronize()
    out["posterior_samples"] = {"draws": 64, "iterations": its, "ms": round((time.perf_counter() - t0) * 1e3, 1),
                                "precond": "learned", "tol": 1e-6}
    del me, mt, xs
    return out


def lbfgs_fit_leg(max_steps=60):
    """Maximum-likelihood fit of the non-stationary model on 150 x 150 x 36
    (810,000 nodes) observed at 0.5 % of nodes plus a sensor track of 2,000
    points per step, data simulated at the known parameters (seed 3); L-BFGS on
    the exact adjoint gradients from a start with every parameter of the
    diffusion, advection and noise perturbed (the initial-field parameters held)."""
    import torch
    from spdepy_gb300.optim import Optimize
    from spdepy_gb300.workloads import build_model, sensor_track_advection_diffusion, simulate
    w = sensor_track_advection_diffusion()
    mod = build_model(w, "mixed")
    simulate(mod, w, seed=4)
    truth = w.par.copy()
    rng = np.random.default_rng(5)
    x0 = truth + rng.normal(0.0, 0.2, truth.size)
    fix = np.arange(truth.size - 5, truth.size - 1)  # initial-field model
    x0[fix] = truth[fix]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = Optimize(mod.logLike).fit(x0=x0, stepType="lbfgs", max_steps=max_steps, fix=fix)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    free = np.setdiff1d(np.arange(truth.size), fix)
    err = float(np.linalg.norm(res["x"][free] - truth[free]) / np.linalg.norm(truth[free]))
    # the same gradient at the truth by Hutchinson traces (64 Rademacher probes)
    # with learned-PCG solves, against the exact selected-inversion gradient
    from spdepy_gb300.precond import LearnedPreconditioner, system_maker
    from spdepy_gb300.workloads import nonstationary_advection_diffusion
    wt = nonstationary_advection_diffusion(M=100, N=100, T=12)
    mt = build_model(wt, "iterative")
    lp = LearnedPreconditioner(seed=0)
    lp.train(system_maker(wt, mt), steps=2000, probes=4, lr=3e-3, seed=1)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    _, j_exact = mod.logLike(truth, grad=True)
    torch.cuda.synchronize()
    t_exact = time.perf_counter() - t1
    np.random.seed(11)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    j_h, its = mod.logLikeGradPCG(truth, precond=lp, nh1=64, tol=1e-6)
    torch.cuda.synchronize()
    t_h = time.perf_counter() - t1
    hutch = {"probes": 64, "pcg": "learned (2,000 systems at 100x100x12)", "pcg_iterations": its,
             "seconds": round(t_h, 3), "exact_seconds": round(t_exact, 3),
             "rel_err_vs_exact": float(np.abs(j_h - j_exact)[free].max() / np.abs(j_exact[free]).max())}
    err0 = float(np.linalg.norm(x0[free] - truth[free]) / np.linalg.norm(truth[free]))
    return {"workload": w.name + f" ({w.grid.n} nodes, {w.idx.size} observations)", "method": "L-BFGS, exact gradient",
            "free_parameters": int(free.size), "iterations": res["nit"], "evaluations": res["nfev"],
            "seconds": round(secs, 2), "rel_param_error_start": err0, "rel_param_error_fit": err,
            "f_start": float(mod.logLike(x0, grad=False)), "f_fit": float(res["fun"]),
            "f_truth": float(mod.logLike(truth, grad=False)),
            "grad_inf_fit": float(np.abs(np.asarray(res["jac"])[free]).max()), "hutchinson_pcg_gradient": hutch}


def config2_leg():
    """Stationary advection-diffusion, 100 x 100 x 24 (240,000 nodes), 2,000
    observations per step, sigma = 0.05, bc 1: the mixed plan (FP32 factor with
    3xTF32 products, FP64 pivots and refinement) against the FP64 plan for logL,
    the exact gradient and 256 samples drawn from the same z."""
    import torch
    from spdepy_gb300.workloads import build_model, simulate, stationary_advection_diffusion
    w = stationary_advection_diffusion()
    out = {"workload": w.name + f" ({w.grid.n} nodes, {w.idx.size} observations)"}
    res = {}
    for prec in ("fp64", "mixed"):
        mod = build_model(w, prec)
        if prec == "fp64":
            simulate(mod, w)
        else:
            mod.initFit(w.y, idx=w.idx)
        mod.logLike(w.par, grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f, jac = mod.logLike(w.par, grad=True)
        torch.cuda.synchronize()
        t_eval = time.perf_counter() - t0
        mod._assemble(w.par)
        mod.plan.factor(False, 0.0)
        z = torch.as_tensor(np.random.default_rng(7).normal(size=(w.grid.n, 256))).cuda()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x = mod.plan.sample(z)
        torch.cuda.synchronize()
        res[prec] = (f, jac, x.cpu().numpy(), t_eval, time.perf_counter() - t0)
        del mod, x, z
    f64, j64, x64, t64, s64 = res["fp64"]
    fmx, jmx, xmx, tmx, smx = res["mixed"]
    out.update({"rel_dlogL": abs(fmx - f64) / abs(f64), "abs_dlogL": abs(fmx - f64) * float(w.idx.size),
                "evals_per_s": {"fp64": round(1.0 / t64, 4), "mixed": round(1.0 / tmx, 3)}, "rel_dgrad": float(np.abs(jmx - j64).max() / np.abs(j64).max()),
                "rel_dsamples": float(np.abs(xmx - x64).max() / np.abs(x64).max()),
                "eval_s": {"fp64": round(t64, 3), "mixed": round(tmx, 3)},
                "sample256_s": {"fp64": round(s64, 3), "mixed": round(smx, 3)}})
    return out


def replica_throughput(local_ms, steps, world, dist=None, device="cpu"):
    """Whole-job evaluations/s of `world` independent replicas that each ran
    `steps` evaluations in `local_ms`: the job time is the slowest rank's (max
    over ranks), returned with the throughput."""
    ms = float(local_ms)
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return world * steps / (ms / 1e3), ms


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU path (the oracle port) timed on the host
    cores.  A step is one evaluation of the 30 x 30 x 24 sub-grid of the same
    model (about 15 s of CPU work); W warm-up steps (at most two) run the
    20 x 20 x 24 sub-grid, then K timed steps (stopping after 240 s of timed work),
    then one evaluation of the 50 x 50 x 24 sub-grid (60,000 nodes), the largest
    that fits the time budget.  `value` scales the 50 x 50 x 24 cost linearly in
    nodes to one evaluation of the benchmarked workload; `ms_per_step` is the
    measured time of a timed step."""
    if rank != 0:
        return
    M, N, T = (int(v) for v in args.size.split(","))
    small, step, large = _cpu_ladder(((20, 20), (30, 30), (50, 50)))
    warm = [_time_ladder([small], k)[0] for k in range(min(args.warmup, 2))]
    t0 = time.perf_counter()
    timed = []
    for k in range(args.steps):
        timed.append(_time_ladder([step], 100 + k)[0][1])
        if time.perf_counter() - t0 > 240.0:
            break
    big = _time_ladder([large], 7)[0]
    points = ([(warm[-1][0], warm[-1][1])] if warm else []) + [(step[0], float(np.mean(timed))), big]
    cb = _cpu_figures(points, M * N * T, len(timed))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "evals/s", "n_gpus": args.gpus,
            "steps": len(timed), "warmup": len(warm), "ms_per_step": 1e3 * float(np.mean(timed)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"nonstationary advection-diffusion {M}x{N}x{T}",
                       "step": f"one reference-path evaluation (logL + Hutchinson gradient, nh1=100) of the "
                               f"{step[0]}-node 30x30x24 sub-grid; ms_per_step is its measured time",
                       "value": f"the {big[0]}-node 50x50x24 sub-grid's seconds per evaluation ({big[1]:.1f} s) "
                                f"scaled linearly in nodes to the {M * N * T}-node workload"},
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "evals/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--size", default="200,200,24")
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="timed evaluations of the plain FP64 plan (the metric's denominator); 0 skips it")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-pcg", action="store_true")
    ap.add_argument("--pcg-only", action="store_true", help="run only the learned-PCG leg and print its record")
    ap.add_argument("--pcg-train-steps", type=int, default=5000)
    ap.add_argument("--pcg-size", default="400,400,48")
    ap.add_argument("--fit", action="store_true", help="also run the L-BFGS fit on the sensor-track workload")
    ap.add_argument("--no-config2", action="store_true",
                    help="skip the mixed-vs-FP64 comparison on the stationary 100x100x24 model")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.pcg_only:
        from spdepy_gb300 import build as b
        b.build()
        size = tuple(int(v) for v in args.pcg_size.split(","))
        print(json.dumps({"learned_pcg": learned_pcg_leg(args.pcg_train_steps, size)}))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from spdepy_gb300 import _native as nat
    from spdepy_gb300 import build as b
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion, simulate
    b.build()
    M, N, T = (int(v) for v in args.size.split(","))
    w = nonstationary_advection_diffusion(M, N, T)
    mod = build_model(w, args.precision)
    simulate(mod, w)
    plan = mod.plan
    plan.set_obs(w.grid.obs_nodes(w.idx))
    canon = mod.canonical(w.par)
    y_dev = torch.as_tensor(w.y).cuda()
    info = plan.info()

    def evaluate():
        return plan.loglike(canon, y_dev, 1)

    for _ in range(args.warmup):
        evaluate()
    torch.cuda.synchronize()
    L = nat.lib()
    L.spde_plan_read_profile(plan.h, None, None, None, 1)
    L.spde_plan_set_profiling(plan.h, 2)  # events around the tensor-core products only
    launches0 = plan.info().launches
    clocks = Clocks()
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        f, jac = evaluate()
    e1.record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evals_per_s, ms = replica_throughput(e0.elapsed_time(e1), args.steps, world, dist, "cuda")
    clk = clocks.stop()
    launches = plan.info().launches - launches0
    pms, pfl, pct = (np.zeros(10), np.zeros(10), np.zeros(10, dtype=np.int64))
    L.spde_plan_read_profile(plan.h, pms.ctypes.data, pfl.ctypes.data, pct.ctypes.data, 1)
    L.spde_plan_read_sites(plan.h, None, None, None, 1)
    # one more pass with every launch timed, for the split by kernel class and call
    # site: on one pipeline, so that each launch's time is its own and not the
    # other pipeline's contention (then back to two, with a warm-up evaluation)
    nat.check(L.spde_plan_set_pipelines(plan.h, 1), plan.h)
    L.spde_plan_set_profiling(plan.h, 1)
    evaluate()
    L.spde_plan_set_profiling(plan.h, 0)
    cms, cfl, cct = (np.zeros(10), np.zeros(10), np.zeros(10, dtype=np.int64))
    L.spde_plan_read_profile(plan.h, cms.ctypes.data, cfl.ctypes.data, cct.ctypes.data, 1)
    nat.check(L.spde_plan_set_pipelines(plan.h, 2), plan.h)
    evaluate()
    sms, sfl, stl = np.zeros(18), np.zeros(18), np.zeros(18, dtype=np.int64)
    L.spde_plan_read_sites(plan.h, sms.ctypes.data, sfl.ctypes.data, stl.ctypes.data, 1)
    site_names = ["", "factor_panel_solve", "factor_panel_update", "factor_schur", "fwd_diag", "fwd_below", "fwd_border",
                  "bwd_border", "bwd_diag", "bwd_above", "inv_x_solve", "inv_x_update", "inv_zbs", "inv_xj", "inv_zrj",
                  "inv_zjj", "inv_zjj2", "inv_zss"]
    sites = {site_names[i]: {"ms": round(float(sms[i]), 3),
                             "tflops": round(float(sfl[i] / max(sms[i], 1e-9) / 1e9), 2),
                             "tiles": int(stl[i])} for i in range(1, 18) if sms[i] > 0}

    # end to end through the public API: host data in, host objective/gradient out
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        mod.logLike(w.par, grad=True)
    torch.cuda.synchronize()
    n_e2e = max(1, args.steps // 2)
    e2e_rate, _ = replica_throughput((time.perf_counter() - t0) * 1e3, n_e2e, world, dist, "cuda")

    # posterior-style sampling: factor + 256-column P L^-T z, as Model.sample does
    z = torch.randn(w.grid.n, 256, dtype=torch.float64, device="cuda")
    mod._assemble(w.par)
    plan.factor(False, 0.0)
    plan.sample(z)
    torch.cuda.synchronize()
    s0 = time.perf_counter()
    plan.factor(False, 0.0)
    plan.sample(z)
    torch.cuda.synchronize()
    samples_per_s = 256.0 / (time.perf_counter() - s0)

    nobs_total = float(w.idx.size)  # m r, the objective's normalisation (r = 1)
    fp64 = None
    dgemm = _dgemm_tflops(torch)
    if args.fp64_steps > 0:
        # the plain FP64 plan on the same workload: the metric's denominator
        m64 = build_model(w, "fp64")
        m64.initFit(w.y, idx=w.idx)
        m64._ensure_model()
        m64.plan.set_obs(w.grid.obs_nodes(w.idx))
        c64 = m64.canonical(w.par)
        m64.plan.loglike(c64, y_dev, 0)  # warm-up: both factorisations and the solve, no inversion
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.fp64_steps):
            f64, j64 = m64.plan.loglike(c64, y_dev, 1)
        torch.cuda.synchronize()
        t64 = (time.perf_counter() - t0) / args.fp64_steps
        dense_flops = 2.0 * (info.factor_flops + info.selinv_flops)
        fp64 = {"evals_per_s": 1.0 / t64, "s_per_eval": t64, "steps": args.fp64_steps, "f": f64,
                "mixed_speedup": evals_per_s * t64,
                "rel_dlogL_mixed_vs_fp64": abs(f - f64) / abs(f64),
                "abs_dlogL_mixed_vs_fp64": abs(f - f64) * nobs_total,
                "rel_dgrad_mixed_vs_fp64": float(np.abs(jac - j64).max() / np.abs(j64).max()),
                "dense_tflops": dense_flops / t64 / 1e12, "dgemm_cublas_tflops": dgemm,
                "frac_of_dgemm": (dense_flops / t64 / 1e12) / dgemm if dgemm else None,
                "note": "one FP64-plan evaluation after a warm-up without inversion; abs_dlogL is |f - f64| "
                        "times m r, the difference in the log-likelihood itself; dense_tflops counts the two "
                        "factorisations' and two inversions' algorithmic flops"}
        del m64

    peaks, peak_src = _peaks()
    # dominant kernel: the tensor-core tiled product (profile class 9), timed
    # inside a step of several hundred ms: the sustained bf16 figure is its peak
    tc_ms = pms[9] / args.steps
    tc_launch_avg_ms = pms[9] / max(1, pct[9])
    tc_flops_per_launch = pfl[9] / max(1, pct[9])
    achieved = tc_flops_per_launch / (tc_launch_avg_ms / 1e3) / 1e12
    peak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0)))
    tf32 = _tf32_tflops(torch)
    if rank != 0:
        return
    cb = None if (args.no_cpu or world > 1) else cpu_baseline(w.grid.n)  # rank 0 at N = 1 only
    pcg = None if args.no_pcg else learned_pcg_leg(args.pcg_train_steps)
    fit = lbfgs_fit_leg() if args.fit else None
    c2 = None if args.no_config2 else config2_leg()
    nobs = int(w.idx.size)
    line = {
        "metric": METRIC, "value": evals_per_s, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": w.name, "nodes": int(w.grid.n), "parameters": int(w.par.size),
                   "parameters_note": "107 parameters (B-spline kappa, gamma, vx, vy: 25 each; lambda; log sigma; "
                                      "4 initial-field parameters; log tau), a superset of the ~55 the "
                                      "configuration states (it ties kappa and gamma to constants)",
                   "observations": nobs,
                   "precision": args.precision, "gradient": "exact (selected inversion + adjoint)",
                   "l2": "inputs and factor arenas far larger than L2 (factor %.1f GB)" % (info.bytes_factor / 1e9),
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_rate, "unit": "evals/s", "h2d_bytes_per_step": nobs * 8 + int(canon.size) * 8,
                "d2h_bytes_per_step": int(canon.size) * 8 + 8},
        "samples_per_s": samples_per_s,
        "gpu_launches": int(launches),
        "roofline": {"bound": "tensor", "kernel": "tc_pair_kernel + tc_gemm_kernel (3xTF32 tiled products: factor and "
                                                  "inverse updates; cluster pairs on 256x256 tiles, single CTAs below)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "peak_source": f"bf16 dense, sustained, {peak_src}",
                     "traffic": TC_DRAM_BYTES_PER_FLOP * tc_flops_per_launch,
                     "traffic_source": "ncu dram bytes per flop of the largest captured pair launch "
                                       "(100x100x24), scaled by this run's flops per launch",
                     "launches_per_step": float(pct[9] / args.steps),
                     "note": "CUDA events around each tensor-core launch in the timed region, while the Q and "
                             "Q + tau S^T S pipelines run concurrently on two streams (a launch's time includes "
                             "waiting for SMs held by the other pipeline); achieved_one_pipeline and the per-class "
                             "split below come from one extra evaluation on one pipeline with every launch timed",
                     "achieved_one_pipeline": float(cfl[9] / max(cms[9], 1e-9) / 1e9),
                     "share_of_step": tc_ms / (ms / args.steps),
                     "tf32_cublas_tflops": tf32,
                     "frac_of_3xtf32": achieved / (tf32 / 3.0) if tf32 else None},
        "profile_ms_per_step": {k: float(cms[i]) for i, k in enumerate(
            ["memset", "extend_add", "diag_block", "product_cuda_cores", "fwd_gather", "bwd_gather", "inv_gather",
             "transpose", "inv_extract", "product_tensor_cores"])},
        "algorithmic": {"factor_tflop": info.factor_flops / 1e12, "selinv_tflop": info.selinv_flops / 1e12,
                        "nnz_L": info.nnz_l},
        "gemm_sites": sites,
        "objective": f, "clocks": clk, "cpu_baseline": cb, "fp64_plain": fp64, "learned_pcg": pcg, "lbfgs_fit": fit, "stationary_100x100x24": c2,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
