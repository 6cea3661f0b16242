#!/usr/bin/env python
"""Benchmark of the GB300 ACHR sampler: chain-steps/s on the genome-scale workload.

Workload ("genome"): seeded synthetic model 2766 metabolites x 3742 reactions
(each reaction touches 2-6 metabolites, coefficients in {-2,-1,1,2}, 30%
irreversible, 150 exchange reactions bounded +-20), 7484 = 2n warmup points,
100,000 chains x 2000 steps, plain ACHR in FP64 with the reference's
semantics.  One "step" of this benchmark is one full sampling launch of that
workload (2e8 chain-steps).  The warmup matrix (224 MB) exceeds the 129 MB L2,
so no explicit L2 flush is done between timed launches.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload genome|small]

Prints one JSON line on rank 0.  --impl reference times the CPU restatement of
the reference's sampling loop (the oracle, OpenMP over chains, all host
threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import re
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "chain-steps/s"
WORKLOADS = {
    # name: (spec attribute, chains, steps)
    "genome": ("GENOME", 100_000, 2000),
    "small": ("SMALL", 1000, 1000),
    "large": ("LARGE", 262_144, 5000),
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch64"], default="genome")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ess", action="store_true", help="skip the bounded min-ESS/s and R-hat leg")
    ap.add_argument("--no-exact-leg", action="store_true", help="skip the short exact-warmup comparison")
    ap.add_argument("--ess", type=int, nargs=4, metavar=("CHAINS", "BURNIN", "SEGMENTS", "STEPS"),
                    help="min-ESS/s and max R-hat from trace snapshots: CHAINS chains, BURNIN steps, then SEGMENTS "
                         "snapshots STEPS steps apart")
    ap.add_argument("--gemm", type=int, metavar="CHAINS", help="time the tensor-core GEMM alone at this N")
    ap.add_argument("--null-report", action="store_true", help="null-space set-up time and basis quality")
    ap.add_argument("--cli", action="store_true",
                    help="wall time of the drop-in CLI on the 72 x 95 fixture; with --chains P, at genome scale "
                         "(the bench model as MPS and %%f CSV, P points x 2000 steps)")
    ap.add_argument("--learned", type=int, nargs=4, metavar=("CHAINS", "BURNIN", "SEGMENTS", "STEPS"),
                    help="learned-preconditioned hit-and-run against plain ACHR on this ESS schedule")
    ap.add_argument("--train-chains", type=int, default=65536)
    ap.add_argument("--train-burnin", type=int, default=2000)
    ap.add_argument("--train-snapshots", type=int, default=8)
    ap.add_argument("--train-gap", type=int, default=250)
    ap.add_argument("--precond-rank", type=int, default=256, help="rank of the learned preconditioner")
    ap.add_argument("--iters", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=0.01)
    ap.add_argument("--pool", type=int, default=16384)
    ap.add_argument("--start", choices=["warmup", "centre"], default="warmup",
                    help="ESS runs: chains start at random warmup points (over-dispersed, default) or at the centre")
    ap.add_argument("--minibatch", action="store_true", help="train on minibatches instead of the full covariance")
    ap.add_argument("--refine", type=int, default=0,
                    help="re-fit the preconditioner this many times on the learned sampler's own samples")
    ap.add_argument("--large-chains", type=int, default=262_144, help="chains of the large workload")
    ap.add_argument("--large-steps", type=int, default=200, help="timed steps of the large workload")
    ap.add_argument("--threads-per-chain", type=int, default=0, help="chain-kernel block size (0: by model size)")
    ap.add_argument("--warmup-form", choices=["percent_f", "exact"], default="percent_f",
                    help="warmup points as the reference's %%f CSV holds them, or exact FP64 chord points")
    ap.add_argument("--chains", type=int, default=0, help="override the workload's chain count (0: its own)")
    ap.add_argument("--bracket-pass", type=int, choices=[0, 1], default=0,
                    help="0: ratio-test brackets formed with the direction; 1: a separate pass")
    ap.add_argument("--reproject-form", type=int, default=None, choices=[0, 1, 2, 3],
                    help="the library's reprojection form (default: chosen from the inputs)")
    ap.add_argument("--profile-case", type=int, nargs=2, metavar=("CHAINS", "STEPS"),
                    help="run two launches of CHAINS x STEPS of the workload and print their times (ncu captures)")
    return ap.parse_args()


def sampler_options(args):
    """Chain-kernel options from the command line (defaults: chosen by the library)."""
    o = {"threads_per_chain": args.threads_per_chain, "bracket_pass": args.bracket_pass}
    if args.reproject_form is not None:
        o["reproject_form"] = args.reproject_form
    return o


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic_per_chain_step(workload, segmented=False):
    """DRAM bytes per chain-step from the committed ncu summary of the chain kernel (the segmented
    instantiation's figure when the run reprojected through the batched passes)."""
    p = ROOT / "profiles" / f"chain_kernel_{workload}.md"
    if not p.exists():
        return None
    key = "dram_bytes_per_chain_step_segmented" if segmented else "dram_bytes_per_chain_step"
    m = re.search(key + r":\s*([0-9.eE+-]+)", p.read_text())
    return float(m.group(1)) if m else None


def gpu_null_space_fn(pkg):
    """Null-space basis of a dense matrix through the library (cuSOLVER), for warmup generation."""
    def null_space(SF):
        r, c = np.nonzero(SF)
        m = pkg.HostModel(SF.shape[1], SF.shape[0], r, c, SF[r, c], np.full(SF.shape[1], -1.0),
                          np.full(SF.shape[1], 1.0))
        with pkg.Sampler(m, np.zeros((SF.shape[1], 1))) as tmp:
            return tmp.null_space()
    return null_space


def percent_f(pkg, warm, tag):
    """The warmup matrix as the reference reads it: written with "%f" (one line per reaction, as
    VFWarmup/createWarmupPtsGLPK.c:289-297 writes it) and read back (ACHRcu/ACHRCuda.cu:675-689),
    through the library's own writer and reader."""
    path = Path("/tmp") / f"achr_bench_{tag}_warmup.csv"
    pkg.write_points_csv(path, warm)
    out = pkg.read_warmup_csv(path, warm.shape[0])
    path.unlink()
    return out


def build_inputs(workload, pkg, synth, null_space=None, warmup_form="exact"):
    """Model arrays, dense S and warmup points (numpy; identical for both arms).
    Cached under /tmp so the two arms of one run share the set-up work.  warmup_form
    "percent_f" rounds the points to six decimals as the reference's CSV holds them."""
    spec_name, P, T = WORKLOADS[workload]
    spec = getattr(synth, spec_name)
    cache = Path("/tmp") / f"achr_bench_{workload}_{spec.seed}_{warmup_form}_v2.npz"
    row, col, val, lb, ub = synth.make_model(spec)
    S = synth.dense(spec.n_mets, spec.n_rxns, row, col, val)
    W = 2 * spec.n_rxns
    if cache.exists():
        warm = np.load(cache)["warm"]
    else:
        warm = synth.interior_chord_warmup(S, lb, ub, W, seed=spec.seed + 17, null_space=null_space)
        if warmup_form == "percent_f":
            warm = percent_f(pkg, warm, f"{workload}_{spec.seed}")
        np.savez(cache, warm=warm)
    model = pkg.HostModel(spec.n_rxns, spec.n_mets, row, col, val, lb, ub)
    return spec, model, S, warm, P, T


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.gpu_index = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r for r in csv.reader(io.StringIO(out)) if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_chains_for(prob, T, seed, target_s, threads):
    """Chains (a multiple of the thread count) whose T steps take about target_s on the oracle.

    A first short call pays the one-time costs (thread start-up, first touch of the warmup
    matrix); the probe then doubles its chain count until it runs for at least 0.3 s, so that
    the per-call overhead does not inflate the estimated cost of a chain-step."""
    prob.sample(seed, threads, 5, chain_offset=2 * 10**9, threads=threads)
    steps = min(T, 100)
    chains = threads
    while True:
        t0 = time.perf_counter()
        prob.sample(seed, chains, steps, chain_offset=10**9, threads=threads)
        el = time.perf_counter() - t0
        if el >= 0.3 or chains * steps * 1.0 >= 1e9:
            break
        chains *= 2
    rate = chains * steps / el  # chain-steps per second
    rounds = max(1, int(target_s * rate / (T * threads)))
    return threads * rounds


def cpu_baseline(oracle, model, warm, N, T, seed, target_s):
    """Time the oracle (all host threads) on a bounded chain sample of the workload."""
    threads = os.cpu_count() or 1
    prob = oracle.Problem(model, warm, N)
    P = cpu_chains_for(prob, T, seed, target_s, threads)
    t0 = time.perf_counter()
    _, st = prob.sample(seed, P, T, threads=threads)
    el = time.perf_counter() - t0
    return {"value": st["accepted"] / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{P} chains x {T} steps of the same workload ({st['accepted']} chain-steps, {el:.1f} s)"}


def oracle_null_space(S):
    """Null-space basis by the reference's rule (S^T S spectrum, cutoff n*s0*2.2204e-16), numpy eigh."""
    n = S.shape[1]
    lam, V = np.linalg.eigh(S.T @ S)
    tol = n * np.abs(lam).max() * 2.2204e-16
    keep = np.abs(lam) < tol
    return V[:, keep] if keep.any() else V


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    import __graft_entry__ as ge
    import oracle

    pkg = ge.load_package()
    import importlib
    synth = importlib.import_module("achr_gb300.synthetic")
    oracle.build()
    spec, model, S, warm, P, T = build_inputs(args.workload, pkg, synth, warmup_form=args.warmup_form)
    if args.chains:
        P = args.chains
    N = oracle_null_space(S)
    threads = os.cpu_count() or 1
    prob = oracle.Problem(model, warm, N)
    # each step: a bounded chain sample of the workload sized to ~8 s
    Pstep = min(P, cpu_chains_for(prob, T, args.seed, 8.0, threads))
    for w in range(args.warmup):
        prob.sample(args.seed + w, threads, min(T, 50), threads=threads)
    times, acc = [], 0
    for k in range(args.steps):
        t0 = time.perf_counter()
        _, st = prob.sample(args.seed + 100 + k, Pstep, T, chain_offset=k * Pstep, threads=threads)
        times.append(time.perf_counter() - t0)
        acc += st["accepted"]
    total = sum(times)
    value = acc / total
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {spec.n_mets}x{spec.n_rxns} synthetic model, W={warm.shape[1]}, "
                               f"{P} chains x {T} steps (CPU step = {Pstep} chains x {T} steps), "
                               f"warmups {args.warmup_form}",
                   "parallelism": f"openmp{threads}"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{Pstep} chains x {T} steps per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ess_leg(pkg, synth, args, genome_inputs):
    """The metric's second half (min-ESS/s and R-hat), bounded to about a minute of the default run.

    * small 72 x 95 model: plain ACHR, isotropic hit-and-run, PCA-only and learned directions
      (learned_study) on a schedule where the chains reach R-hat < 1.01: 1000 chains from random
      warmup points, 100,000 burn-in steps, 200 draws 1000 steps apart; training on 65,536 chains
      x (2000 + 8 x 250) plain steps, rank 4 (the basis has 9 directions), 2000 full-batch Adam steps.
    * the bench's own genome model: plain ACHR, 512 chains from random warmup points, 20,000 burn-in
      steps, 40 draws 500 steps apart (far from R-hat < 1.01 at this length; reported as measured).
    min-ESS/s divides the smallest bulk ESS over the moving fluxes by the device time of the
    sampling launches (burn-in included)."""
    import importlib

    import torch

    diag = importlib.import_module("achr_gb300.diagnostics")
    t0 = time.perf_counter()
    out = {}
    spec_s, model_s, _, warm_s, _, _ = build_inputs("small", pkg, synth, warmup_form=args.warmup_form)
    with pkg.Sampler(model_s, warm_s) as smp:
        res = learned_study(pkg, diag, smp, warm_s, seed=args.seed, train=(65536, 2000, 8, 250), rank=4, iters=2000,
                            lr=0.01, batch=4096, pool=16384, schedule=(1000, 100000, 200, 1000))
    res.pop("value")
    out["small"] = {"model": f"{spec_s.n_mets}x{spec_s.n_rxns}", **res}
    spec, model, warm = genome_inputs
    M, B, K, L = 512, 20000, 40, 500
    stream = torch.cuda.current_stream().cuda_stream
    with pkg.Sampler(model, warm) as smp:
        draws, ms, steps = ess_trace(smp, M, B, K, L, args.seed + 101, stream,
                                     starts=dispersed_starts(warm, M, args.seed + 5))
    summ = diag.summarize(draws, exclude=pinned_reactions(warm))
    out["genome_plain"] = {"model": f"{spec.n_mets}x{spec.n_rxns}",
                           "schedule": {"chains": M, "burnin": B, "draws": K, "gap": L,
                                        "starts": "random warmup points"},
                           "min_ess_per_s": summ["min_ess"] / (ms * 1e-3), "min_ess": summ["min_ess"],
                           "max_rhat": summ["max_rhat"], "rhat_below_1.01": summ["max_rhat"] < 1.01,
                           "median_rhat": summ["median_rhat"], "sampling_ms": ms,
                           "chain_steps_per_s": steps / (ms * 1e-3)}
    out["seconds"] = time.perf_counter() - t0
    return out


def run_gpu(args):
    rank, world, local = dist_info()
    import torch

    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device")
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import importlib

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    synth = importlib.import_module("achr_gb300.synthetic")
    spec, model, S, warm, P, T = build_inputs(args.workload, pkg, synth, warmup_form=args.warmup_form)
    if args.chains:
        P = args.chains
    n = spec.n_rxns
    sharding = importlib.import_module("achr_gb300.sharding")
    chain_base, _ = sharding.chain_block(rank, world, P)  # weak scaling: every rank runs its own P chains

    t_setup = time.perf_counter()
    smp = pkg.Sampler(model, warm, **sampler_options(args))
    setup_s = time.perf_counter() - t_setup
    stream = torch.cuda.current_stream()
    out = torch.empty((n, P), dtype=torch.float64, device="cuda")

    stats = None
    for w in range(args.warmup):
        st = smp.sample_device(P, T, out.data_ptr(), P, stream.cuda_stream, seed=args.seed + w,
                               chain_offset=chain_base, with_stats=(w == args.warmup - 1))
        stats = st or stats
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.synchronize()
    evs[0].record(stream)
    timed = []  # per step: the library's own split of its device time (chain kernel / batched reprojection)
    for k in range(args.steps):
        timed.append(smp.sample_device(P, T, out.data_ptr(), P, stream.cuda_stream, seed=args.seed + 1000 + k,
                                       chain_offset=chain_base, with_stats=True))
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    per_launch = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    ms = sum(per_launch) / args.steps
    if world > 1:
        ms = sharding.max_over_ranks(ms, device="cuda")
        torch.distributed.barrier()
    chain_steps = P * T
    value = world * chain_steps / (ms * 1e-3)

    # Roofline of the dominant kernel, the chain kernel: its algorithmic bytes over its own device
    # time (CUDA events around its launches on the launch stream, inside the library).
    peak, peak_kind = load_peaks()
    alg_bytes = synth.ideal_bytes_per_chain_step(n) * chain_steps
    chain_ms = sum(s["chain_ms"] for s in timed) / len(timed)
    launches = max(1, int(round(sum(max(1, s["segments"]) for s in timed) / len(timed))))
    achieved = alg_bytes / (chain_ms * 1e-3) / 1e9
    tpcs = profile_traffic_per_chain_step(args.workload, segmented=any(s["segments"] > 0 for s in timed))
    roofline = {"bound": "hbm", "kernel": "achr_chain_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": (tpcs * chain_steps) if tpcs is not None else None,
                "peak_source": f"{peak_kind} hbm_gbs (burst copy)", "algorithmic_bytes_per_step": alg_bytes,
                "kernel_ms_per_step": chain_ms, "kernel_launches_per_step": launches,
                "whole_step_frac": alg_bytes / (ms * 1e-3) / 1e9 / peak}
    reproj = None
    rms = sum(s["reprojection_ms"] for s in timed) / len(timed)
    if rms > 0:
        tpk, tpk_kind = load_tensor_peak()
        rfl = sum(s["reprojection_flops"] for s in timed) / len(timed)
        reproj = {"form": "deferred batched (three BF16 split products on the tensor cores, FP32 passes)",
                  "ms_per_step": rms, "share_of_step": rms / ms,
                  "chain_passes_per_reprojection": timed[-1]["reprojection_passes"] / max(1, timed[-1]["reprojections"]),
                  "gemms_per_step": timed[-1]["reprojection_gemms"], "gemm_tflop_per_step": rfl / 1e12,
                  "tensor_tflops_over_pass_time": rfl / (rms * 1e-3) / 1e12, "tensor_peak_tflops": tpk,
                  "tensor_peak_source": tpk_kind}

    # End to end through the public API with host buffers: set-up from pinned host
    # model + warmup (H2D, null space, centre), sampling, D2H of every point.
    e2e = None
    if not args.no_e2e:
        warm_pinned = torch.from_numpy(np.asfortranarray(warm).T.copy()).pin_memory()  # (W, n) = column-major n x W
        host_out = torch.empty((n, P), dtype=torch.float64).pin_memory()
        wnp = warm_pinned.numpy().T  # (n, W) view, Fortran order over pinned memory
        e2e_times = []
        for k in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            with pkg.Sampler(model, wnp, **sampler_options(args)) as s2:
                s2.sample(P, T, seed=args.seed + 2000 + k, chain_offset=chain_base, out=host_out.numpy())
            torch.cuda.synchronize()
            e2e_times.append(time.perf_counter() - t0)
        e2e_s = max(sum(e2e_times) / len(e2e_times), 1e-9)
        if world > 1:  # the job's end-to-end time is the slowest rank's
            e2e_s = sharding.max_over_ranks(e2e_s, device="cuda")
        h2d = warm.size * 8 + len(model.row) * 16 + n * 16
        e2e = {"value": world * chain_steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(n * P * 8), "seconds_per_step": e2e_s}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle

        oracle.build()
        Nb = smp.null_space()
        cpu = cpu_baseline(oracle, model, warm, Nb, T, args.seed, args.cpu_seconds)

    ess = None
    if rank == 0 and world == 1 and not args.no_ess:
        ess = ess_leg(pkg, synth, args, (spec, model, warm))

    # The same workload on exact (unrounded) warmup points, where the reference's residual check
    # never fires: the sampling step alone, for comparison with the %f figure above.
    exact = None
    if rank == 0 and world == 1 and args.warmup_form == "percent_f" and not args.no_exact_leg:
        _, model_x, _, warm_x, _, _ = build_inputs(args.workload, pkg, synth, warmup_form="exact")
        with pkg.Sampler(model_x, warm_x, **sampler_options(args)) as sx:
            sx.sample_device(P, T, out.data_ptr(), P, stream.cuda_stream, seed=args.seed)
            xs = [sx.sample_device(P, T, out.data_ptr(), P, stream.cuda_stream, seed=args.seed + 7000 + k,
                                   with_stats=True) for k in range(3)]
        xms = sum(s["kernel_ms"] for s in xs) / len(xs)
        exact = {"value": chain_steps / (xms * 1e-3), "unit": METRIC, "steps": len(xs), "ms_per_step": xms,
                 "roofline_frac": alg_bytes / (xms * 1e-3) / 1e9 / peak,
                 "reprojections": xs[-1]["reprojections"], "segments": xs[-1]["segments"]}

    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {spec.n_mets}x{spec.n_rxns} synthetic model, W={warm.shape[1]}, "
                               f"{P} chains x {T} steps per GPU, mode=reference, warmups {args.warmup_form}",
                   "global_batch": world * P, "seq_len": T, "parallelism": f"chains sharded over {world} GPU(s)",
                   "l2": "inputs exceed L2 (warmup matrix 224 MB > 129 MB); no flush",
                   "warmups": ("the reference's input form: chord points written with %f and read back, as "
                               "VFWarmup/createWarmupPtsGLPK.c writes them, so the 10-step checks reproject"
                               if args.warmup_form == "percent_f" else "exact FP64 chord points"),
                   "options": sampler_options(args)},
        "gpu_launches": int(sum(s["kernel_launches"] for s in timed)),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "ess": ess,
        "reprojection": reproj,
        "exact_warmups": exact,
        "sampler": {"null_dim": smp.null_dim, "setup_s": setup_s,
                    **({k: stats[k] for k in ("accepted", "rejected", "checks", "reprojections", "stuck_chains",
                                              "exact_evals", "max_residual", "max_bound_violation", "segments",
                                              "reprojection_passes", "reprojection_gemms")}
                       if stats else {})},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    smp.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_profile_case(args):
    """Two launches of a small chain sample of the workload (the second is the one to capture)."""
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    import importlib
    synth = importlib.import_module("achr_gb300.synthetic")
    # the same warmup construction as the workload's own bench run (the large one uses the GPU null space)
    ns = gpu_null_space_fn(pkg) if args.workload == "large" else None
    spec, model, S, warm, _, _ = build_inputs(args.workload, pkg, synth, null_space=ns, warmup_form=args.warmup_form)
    P, T = args.profile_case
    smp = pkg.Sampler(model, warm, **sampler_options(args))
    out = torch.empty((spec.n_rxns, P), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for k in range(2):
        st = smp.sample_device(P, T, out.data_ptr(), P, stream, seed=args.seed + k, with_stats=True)
        print(f"launch {k}: {st['kernel_ms']:.3f} ms, {P * T / (st['kernel_ms'] * 1e-3):.4e} chain-steps/s, "
              f"{st['exact_evals'] / max(1, P * T):.3f} FP64 ratio evaluations per step", flush=True)
    smp.close()
    return 0


def _batch_interior_worker(job):
    """LP interior point of one batch model, in a spawned worker process."""
    import importlib

    import __graft_entry__ as ge

    ge.load_package()
    return importlib.import_module("achr_gb300.synthetic").batch_interior(job)


def run_batch(args):
    """64 synthetic models of uneven size sampled in one CUDA-graph launch.

    Reaction counts log-uniform in [95, 7440], metabolites 0.7 n, the same S and
    bound law, warmup 2n per model, chains per model proportional to n summing
    to 262,144, 1000 steps; each model's chain-kernel configuration comes from
    the autotuner.  Prints one JSON line (not the driver's headline metric)."""
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    import importlib
    synth = importlib.import_module("achr_gb300.synthetic")
    sizes = synth.log_uniform_sizes(64, 95, 7440, seed=64)
    chains_total, T = 262_144, 1000
    weights = np.array(sizes, dtype=np.float64)
    P = np.floor(chains_total * weights / weights.sum()).astype(int)
    P[np.argmax(P)] += chains_total - int(P.sum())

    t_setup = time.perf_counter()
    # interior points by LP in a worker pool (CPU only; spawned before any GPU use)
    interiors = {}
    todo = [(k, n) for k, n in enumerate(sizes)
            if not (Path("/tmp") / f"achr_batch_{n}_{1000 + k}_v1.npz").exists()]
    if todo:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(len(todo), os.cpu_count() or 1)) as pool:
            for k, v0, blocked in pool.imap_unordered(_batch_interior_worker, sorted(todo, key=lambda t: -t[1])):
                interiors[k] = (v0, blocked)
    pkg.lib()

    def gpu_null_space(SF):
        r, c = np.nonzero(SF)
        m = pkg.HostModel(SF.shape[1], SF.shape[0], r, c, SF[r, c], np.full(SF.shape[1], -1.0),
                          np.full(SF.shape[1], 1.0))
        with pkg.Sampler(m, np.zeros((SF.shape[1], 1))) as tmp:
            return tmp.null_space()

    samplers, outs = [], []
    for k, n in enumerate(sizes):
        spec = synth.batch_spec(k, n)
        cache = Path("/tmp") / f"achr_batch_{n}_{spec.seed}_v1.npz"
        row, col, val, lb, ub = synth.make_model(spec)
        if cache.exists():
            warm = np.load(cache)["warm"]
        else:
            S = synth.dense(spec.n_mets, spec.n_rxns, row, col, val)
            warm = synth.interior_chord_warmup(S, lb, ub, 2 * n, seed=spec.seed, null_space=gpu_null_space,
                                               interior=interiors[k])
            np.savez(cache, warm=warm)
        s = pkg.Sampler(pkg.HostModel(n, spec.n_mets, row, col, val, lb, ub), warm, bracket_pass=args.bracket_pass)
        s.autotune()
        samplers.append(s)
        outs.append(torch.empty((n, int(P[k])), dtype=torch.float64, device="cuda"))
    batch_setup_s = time.perf_counter() - t_setup
    stream = torch.cuda.current_stream().cuda_stream
    ptrs = [o.data_ptr() for o in outs]
    counts = [int(p) for p in P]
    for w in range(args.warmup):
        pkg.sample_batch(samplers, counts, min(T, 50), ptrs, counts, stream=stream, seed=args.seed + w)
    clocks = ClockSampler(0)
    clocks.start()
    runs = []
    for k in range(args.steps):
        runs.append(pkg.sample_batch(samplers, counts, T, ptrs, counts, stream=stream, seed=args.seed + 100 + k))
    clk = clocks.stop()
    graph_ms = sum(r[0]["graph_ms"] for r in runs) / len(runs)
    chain_steps = int(P.sum()) * T
    alg = sum(synth.ideal_bytes_per_chain_step(n) * int(p) * T for n, p in zip(sizes, P))
    peak, peak_kind = load_peaks()
    line = {
        "metric": METRIC, "value": chain_steps / (graph_ms * 1e-3), "unit": METRIC, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": graph_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"batch64: 64 synthetic models, n log-uniform in [95, 7440] (sum {sum(sizes)}), "
                               f"{int(P.sum())} chains in total (proportional to n) x {T} steps, one CUDA-graph launch",
                   "threads_per_chain": sorted({s.options.threads_per_chain for s in samplers})},
        "load_imbalance": sum(r[0]["load_imbalance"] for r in runs) / len(runs),
        "model_finish_ms": {"min": min(runs[-1][1]), "median": float(np.median(runs[-1][1])), "max": max(runs[-1][1])},
        "roofline": {"bound": "hbm", "achieved": alg / (graph_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / (graph_ms * 1e-3) / 1e9 / peak, "traffic": None,
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "clocks": clk, "setup_s": batch_setup_s,
        "sampler": {k: runs[-1][0][k] for k in ("accepted", "rejected", "reprojections", "stuck_chains",
                                                 "max_residual", "max_bound_violation")},
    }
    print(json.dumps(line), flush=True)
    for s in samplers:
        s.close()
    return 0


def pinned_reactions(warm):
    """Reactions with one value in every warmup point (blocked, or pinned at a bound)."""
    return np.ptp(warm, axis=1) <= 1e-9 * np.maximum(1.0, np.abs(warm).max(axis=1))


def dispersed_starts(warm, M, seed):
    """Over-dispersed starting points for R-hat: chain p starts at a random warmup point
    (seeded), with the centre accumulator of a fresh chain, (W) * centre of the warmups."""
    import torch

    rng = np.random.default_rng(seed)
    idx = torch.from_numpy(rng.integers(0, warm.shape[1], size=M))
    w = torch.from_numpy(np.ascontiguousarray(warm)).cuda()
    x0 = w[:, idx.cuda()].contiguous()
    a0 = (float(warm.shape[1]) * w.mean(dim=1, keepdim=True)).expand(-1, M).contiguous()
    return x0, a0


def ess_trace(smp, M, B, K, L, seed, stream, starts=None):
    """Chains from the warmup centre (starts None, the reference's start) or from given
    (x0, A0) device states: B burn-in steps, then K segments of L steps
    (achr_sample_resume); the points after every segment are the draws.
    Returns (draws (chains, draws, fluxes), device ms of all launches, chain-steps)."""
    import torch

    n = smp.n
    pts = torch.zeros((n, M), dtype=torch.float64, device="cuda")
    acc = torch.zeros((n, M), dtype=torch.float64, device="cuda")
    trace = torch.empty((K, n, M), dtype=torch.float64, device="cuda")
    if starts is not None:
        pts.copy_(starts[0])
        acc.copy_(starts[1])
    st = smp.sample_resume(M, 0, B, starts is not None, pts.data_ptr(), acc.data_ptr(), M, stream=stream,
                           seed=seed, with_stats=True)
    ms, steps = st["kernel_ms"], st["accepted"]
    for k in range(K):
        st = smp.sample_resume(M, B + k * L, L, True, pts.data_ptr(), acc.data_ptr(), M, stream=stream, seed=seed,
                               with_stats=True)
        ms += st["kernel_ms"]
        steps += st["accepted"]
        trace[k].copy_(pts)
    torch.cuda.synchronize()
    return trace.permute(2, 0, 1).cpu().numpy(), ms, steps


def run_ess(args):
    """min over fluxes of bulk ESS per second of sampling, and max split-R-hat.

    Chains run BURNIN steps from the warmup centre, then SEGMENTS launches of
    STEPS steps each (achr_sample_resume); the points after every segment are
    the draws.  The time is the device time of all launches (burn-in included);
    the trace copies and the diagnostics are not timed."""
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    import importlib
    synth = importlib.import_module("achr_gb300.synthetic")
    diag = importlib.import_module("achr_gb300.diagnostics")
    spec, model, S, warm, _, _ = build_inputs(args.workload, pkg, synth, null_space=gpu_null_space_fn(pkg))
    M, B, K, L = args.ess
    n = spec.n_rxns
    smp = pkg.Sampler(model, warm)
    stream = torch.cuda.current_stream().cuda_stream
    starts = dispersed_starts(warm, M, args.seed + 5) if args.start == "warmup" else None
    draws, ms, acc_steps = ess_trace(smp, M, B, K, L, args.seed, stream, starts=starts)
    t0 = time.perf_counter()
    summ = diag.summarize(draws, exclude=pinned_reactions(warm))
    diag_s = time.perf_counter() - t0
    line = {
        "metric": "min-ESS/s", "value": summ["min_ess"] / (ms * 1e-3), "unit": "effective samples/s",
        "higher_is_better": True, "n_gpus": 1, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {spec.n_mets}x{n}, {M} chains, {B} burn-in steps, {K} draws "
                               f"{L} steps apart, plain ACHR (reference semantics), chains start at "
                               f"{'random warmup points' if args.start == 'warmup' else 'the warmup centre'}"},
        "max_rhat": summ["max_rhat"], "rhat_below_1.01": summ["max_rhat"] < 1.01, "min_ess": summ["min_ess"],
        "median_rhat": summ["median_rhat"], "rhat_q99": summ["rhat_q99"], "median_ess": summ["median_ess"],
        "fluxes": summ["params"], "frozen_fluxes": summ["frozen_params"], "sampling_ms": ms,
        "chain_steps_per_s": acc_steps / (ms * 1e-3), "diagnostics_s": diag_s,
    }
    print(json.dumps(line), flush=True)
    smp.close()
    return 0


def training_samples(smp, d, seed, train, chain_offset=0):
    """Centred samples of the context's current sampler in the preconditioner's coordinates
    (d x P*K, FP32, device): P chains, Tb burn-in steps, then K snapshots Lg steps apart, each
    mapped by achr_null_coords on the tensor cores.  Returns (Y, device ms of the sampling)."""
    import torch

    n = smp.n
    Pt, Tb, Ks, Lg = train
    stream = torch.cuda.current_stream().cuda_stream
    x = torch.zeros((n, Pt), dtype=torch.float64, device="cuda")
    a = torch.zeros_like(x)
    mu = torch.from_numpy(smp.centre()).cuda()
    Y = torch.empty((d, Pt * Ks), dtype=torch.float32, device="cuda")
    st = smp.sample_resume(Pt, 0, Tb, False, x.data_ptr(), a.data_ptr(), Pt, stream=stream, seed=seed,
                           chain_offset=chain_offset, with_stats=True)
    gen_ms = st["kernel_ms"]
    for k in range(Ks):
        st = smp.sample_resume(Pt, Tb + k * Lg, Lg, True, x.data_ptr(), a.data_ptr(), Pt, stream=stream, seed=seed,
                               chain_offset=chain_offset, with_stats=True)
        gen_ms += st["kernel_ms"]
        smp.null_coords(Pt, x.data_ptr(), Pt, Y.data_ptr() + 4 * k * Pt, Pt * Ks, d_mu=mu.data_ptr(), stream=stream)
    del x, a
    Y -= Y.mean(dim=1, keepdim=True)
    return Y, gen_ms


def learned_study(pkg, diag, smp, warm, *, seed, train, rank, iters, lr, batch, pool, schedule, start="warmup",
                  refine=0, full_batch=1):
    """Plain ACHR against hit-and-run along learned directions, with the two ablations that
    isolate the learning, all on one ESS schedule (same chains, same starts, same seed):

      plain      ACHR, the reference's direction law (warmup point minus centre)
      isotropic  hit-and-run along B z, z ~ N(0, I): the preconditioner's basis, no fit
      pca        hit-and-run along the probabilistic-PCA fit of the samples (no Adam)
      learned    hit-and-run along the map trained from that start (achr_precond_train)

    B is the basis of the directions the polytope spans (pinned reactions held fixed).
    Returns a dict of per-sampler min-ESS/s, R-hat and rates, the training record and the
    fallback decision (learned not below R-hat 1.01 while plain is)."""
    import torch

    stream = torch.cuda.current_stream().cuda_stream
    d, n_frozen = smp.precond_dim()
    r = min(rank, max(1, d - 1))
    t0 = time.perf_counter()
    Y, gen_ms = training_samples(smp, d, seed + 7, train)
    ns = Y.shape[1]
    s_pca = torch.zeros(d, dtype=torch.float32, device="cuda")
    U_pca = torch.zeros((d, r), dtype=torch.float32, device="cuda")
    pkg.precond_train(d, r, ns, Y.data_ptr(), ns, s_pca.data_ptr(), U_pca.data_ptr(), stream=stream, iterations=0,
                      batch=min(batch, ns), init=1)
    s_par, U_par = s_pca.clone(), U_pca.clone()
    tst = pkg.precond_train(d, r, ns, Y.data_ptr(), ns, s_par.data_ptr(), U_par.data_ptr(), stream=stream,
                            iterations=iters, batch=min(batch, ns), learning_rate=lr, seed=seed, init=1,
                            full_batch=full_batch)
    refine_rec = []
    for rnd in range(refine):  # re-fit on samples of the learned sampler itself (fresh chain ids)
        smp.precond_pool(r, s_par.data_ptr(), U_par.data_ptr(), pool, seed=seed + 11)
        Y, _ = training_samples(smp, d, seed + 7, train, chain_offset=(rnd + 1) * train[0])
        smp.set_directions(None)
        refine_rec.append(pkg.precond_train(d, r, ns, Y.data_ptr(), ns, s_par.data_ptr(), U_par.data_ptr(),
                                            stream=stream, iterations=iters, batch=min(batch, ns),
                                            learning_rate=lr, seed=seed + rnd + 1, init=0, full_batch=full_batch))
    del Y
    torch.cuda.empty_cache()
    train_s = time.perf_counter() - t0
    s_iso = torch.zeros(d, dtype=torch.float32, device="cuda")
    U_iso = torch.zeros((d, r), dtype=torch.float32, device="cuda")
    M, B, K, L = schedule
    starts = dispersed_starts(warm, M, seed + 5) if start == "warmup" else None
    out = {}
    for name, pars in (("plain", None), ("isotropic", (s_iso, U_iso)), ("pca", (s_pca, U_pca)),
                       ("learned", (s_par, U_par))):
        if pars is None:
            smp.set_directions(None)
        else:
            smp.precond_pool(r, pars[0].data_ptr(), pars[1].data_ptr(), pool, seed=seed + 11)
        draws, ms, steps = ess_trace(smp, M, B, K, L, seed + 101, stream, starts=starts)
        summ = diag.summarize(draws, exclude=pinned_reactions(warm))
        out[name] = {"min_ess_per_s": summ["min_ess"] / (ms * 1e-3), "min_ess": summ["min_ess"],
                     "max_rhat": summ["max_rhat"], "median_rhat": summ["median_rhat"],
                     "rhat_q99": summ["rhat_q99"], "median_ess": summ["median_ess"], "sampling_ms": ms,
                     "chain_steps_per_s": steps / (ms * 1e-3), "frozen_fluxes": summ["frozen_params"]}
    smp.set_directions(None)
    lp, ll = out["plain"], out["learned"]
    # plain ACHR is the fallback: the learned sampler's figure stands only where it passes R-hat
    fallback = ll["max_rhat"] >= 1.01
    return {
        **out,
        "learned_over_plain": ll["min_ess_per_s"] / lp["min_ess_per_s"],
        "learned_over_isotropic": ll["min_ess_per_s"] / out["isotropic"]["min_ess_per_s"],
        "learned_over_pca": ll["min_ess_per_s"] / out["pca"]["min_ess_per_s"],
        "fallback_to_plain": fallback,
        "value": lp["min_ess_per_s"] if fallback else ll["min_ess_per_s"],
        "schedule": {"chains": M, "burnin": B, "draws": K, "gap": L,
                     "starts": "random warmup points" if start == "warmup" else "the warmup centre"},
        "training": {"samples": ns, "basis_dim": d, "rank": r, "null_dim": smp.null_dim, "pinned_reactions": n_frozen,
                     "generation_ms": gen_ms, "full_batch": bool(full_batch), **tst, "refine_rounds": refine_rec,
                     "total_s": train_s},
    }


def run_learned(args):
    """Learned-preconditioned hit-and-run against plain ACHR, by min-ESS/s (see learned_study):
    training on --train-chains x (--train-burnin + --train-snapshots x --train-gap) plain-ACHR
    steps, --iters Adam steps (full batch unless --minibatch), a pool of --pool directions, then the
    ESS schedule --learned CHAINS BURNIN SEGMENTS STEPS for plain, isotropic, PCA-only and learned."""
    import torch  # noqa: F401

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    import importlib
    synth = importlib.import_module("achr_gb300.synthetic")
    diag = importlib.import_module("achr_gb300.diagnostics")
    t_setup = time.perf_counter()
    spec, model, S, warm, _, _ = build_inputs(args.workload, pkg, synth, null_space=gpu_null_space_fn(pkg),
                                              warmup_form=args.warmup_form)
    smp = pkg.Sampler(model, warm)
    tpc = smp.autotune()
    setup_s = time.perf_counter() - t_setup
    res = learned_study(pkg, diag, smp, warm, seed=args.seed,
                        train=(args.train_chains, args.train_burnin, args.train_snapshots, args.train_gap),
                        rank=args.precond_rank, iters=args.iters, lr=args.lr, batch=args.batch, pool=args.pool,
                        schedule=tuple(args.learned), start=args.start, refine=args.refine,
                        full_batch=0 if args.minibatch else 1)
    M, B, K, L = args.learned
    line = {
        "metric": "min-ESS/s", "value": res.pop("value"), "unit": "effective samples/s", "higher_is_better": True,
        "n_gpus": 1, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {spec.n_mets}x{spec.n_rxns}, {M} chains, {B} burn-in steps, {K} "
                               f"draws {L} steps apart, warmups {args.warmup_form}; learned: rank "
                               f"{res['training']['rank']} + diagonal, {args.iters} Adam steps",
                   "threads_per_chain": tpc},
        **res, "setup_s": setup_s,
    }
    print(json.dumps(line), flush=True)
    smp.close()
    return 0


def load_tensor_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        if "bf16_tflops" in d:
            return float(d["bf16_tflops"]), "measured bf16_tflops (cuBLAS, burst)"
    return 1900.0, "fallback"


def fp64_reprojection(S, lb, ub, X):
    """FP64 oracle of one reprojection pass: clip(x - S^T (S S^T)^+ S x), numpy."""
    lam, U = np.linalg.eigh(S @ S.T)
    keep = lam > S.shape[0] * lam.max() * 2.2204e-16
    R = S @ X
    Z = U[:, keep] @ ((U[:, keep].T @ R) / lam[keep][:, None])
    return np.clip(X - S.T @ Z, lb[:, None], ub[:, None])


def run_large(args):
    """Mixed-precision reprojection workload: 5063 x 7440 model, chains reprojected
    every 100 steps by the batched tensor-core reprojection (achr_sample_periodic,
    no per-chain checks), against plain ACHR with the reference's per-chain FP64
    checks on the same chains.  The timed run is a bounded slice of the 5000-step
    workload (--large-steps, default 200 = two reprojections); chain-steps/s does
    not depend on the slice length.  Prints one JSON line."""
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    import importlib
    synth = importlib.import_module("achr_gb300.synthetic")
    t_setup = time.perf_counter()
    spec, model, S, warm, P, T = build_inputs("large", pkg, synth, null_space=gpu_null_space_fn(pkg))
    P = args.large_chains
    period, Tr = 100, args.large_steps
    n = spec.n_rxns
    smp = pkg.Sampler(model, warm, check_period=0, **sampler_options(args))
    tpc = smp.autotune()
    x = torch.zeros((n, P), dtype=torch.float64, device="cuda")
    a = torch.zeros_like(x)
    stream = torch.cuda.current_stream().cuda_stream
    t_op = time.perf_counter()
    smp.reproject(1, x.data_ptr(), P)  # builds (S S^T)^+ and its BF16 split
    operator_s = time.perf_counter() - t_op
    setup_s = time.perf_counter() - t_setup
    smp.sample_periodic(P, period, period, x.data_ptr(), a.data_ptr(), P, stream=stream, seed=args.seed)  # warm-up
    clocks = ClockSampler(0)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    st, rs = smp.sample_periodic(P, Tr, period, x.data_ptr(), a.data_ptr(), P, stream=stream, seed=args.seed + 1)
    ev1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    # Reprojection accuracy against the FP64 oracle on 64 chains: one more
    # segment without reprojection, snapshot, the snapshot moved off the null
    # space by a row-space vector of size 1e-6 (the residual a %f warmup leaves,
    # well above the 1e-9 trigger, so the passes reproject every one of them),
    # then a reprojection of up to four passes.
    smp.sample_resume(P, Tr, period, True, x.data_ptr(), a.data_ptr(), P, stream=stream, seed=args.seed + 1)
    Xs = x[:, :64].cpu().numpy()
    Xs = Xs + S.T @ (1e-6 * np.random.default_rng(args.seed).standard_normal((S.shape[0], 64)))
    x[:, :64].copy_(torch.from_numpy(Xs))
    r1 = smp.reproject(P, x.data_ptr(), P, d_centre_acc=a.data_ptr(), max_rounds=4, stream=stream)
    got = x[:, :64].cpu().numpy()
    ref = fp64_reprojection(S, model.lb, model.ub, Xs)
    moved = float(np.abs(ref - Xs).max())
    err = float(np.abs(got - ref).max())
    smp.close()
    del x, a
    torch.cuda.empty_cache()
    # Plain ACHR on the same chains: per-chain residual check every 10 steps,
    # FP64 reprojection of a chain when it fires (reference semantics).
    plain = pkg.Sampler(model, warm, **sampler_options(args))
    plain.autotune()
    out = torch.empty((n, P), dtype=torch.float64, device="cuda")
    plain.sample_device(P, 20, out.data_ptr(), P, stream=stream, seed=args.seed)
    torch.cuda.synchronize()
    ev0.record()
    pst = plain.sample_device(P, Tr, out.data_ptr(), P, stream=stream, seed=args.seed + 1, with_stats=True)
    ev1.record()
    torch.cuda.synchronize()
    plain_ms = ev0.elapsed_time(ev1)
    plain.close()
    tpeak, tpeak_kind = load_tensor_peak()
    gemm_tflops = rs["gemm_flops"] / (rs["gemm_ms"] * 1e-3) / 1e12 if rs["gemm_ms"] > 0 else None
    peak, peak_kind = load_peaks()
    alg = synth.ideal_bytes_per_chain_step(n) * P * Tr
    line = {
        "metric": METRIC, "value": st["accepted"] / (ms * 1e-3), "unit": METRIC, "n_gpus": 1, "steps": 1,
        "warmup": 1, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (reprojection GEMM: 3 x bf16 split, fp32 accumulate)", "data": "synthetic",
        "config": {"workload": f"large: {spec.n_mets}x{n} synthetic model, W={warm.shape[1]}, {P} chains x {Tr} "
                               f"steps (of {T}), batched tensor-core reprojection every {period} steps, "
                               f"no per-chain checks", "threads_per_chain": tpc},
        "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / (ms * 1e-3) / 1e9 / peak, "peak_source": f"{peak_kind} hbm_gbs"},
        "reprojection": {
            "passes": rs["rounds"], "gemm_ms": rs["gemm_ms"], "total_ms": rs["total_ms"],
            "share_of_run": rs["total_ms"] / ms, "gemm_tflops": gemm_tflops, "tensor_peak_tflops": tpeak,
            "tensor_frac": (gemm_tflops / tpeak) if gemm_tflops else None, "tensor_peak_source": tpeak_kind,
            "residual_before": rs["residual_before"], "residual_after": rs["residual_after"],
            "rank": rs["rank"], "kappa": rs["lambda_max"] / rs["lambda_min"] if rs["lambda_min"] > 0 else None,
            "oracle_check": {"chains": 64, "max_abs_err": err, "max_correction": moved,
                             "rel_err": err / moved if moved > 0 else None,
                             "residual_before": r1["residual_before"], "residual_after": r1["residual_after"],
                             "max_abs_Sv": float(np.abs(S @ got).max())},
            "operator_setup_s": operator_s,
        },
        "plain_reference_semantics": {"value": pst["accepted"] / (plain_ms * 1e-3), "ms": plain_ms,
                                      "checks": pst["checks"], "reprojections": pst["reprojections"],
                                      "max_residual": pst["max_residual"]},
        "sampler": {k: st[k] for k in ("accepted", "rejected", "stuck_chains", "max_residual", "max_bound_violation")},
        "clocks": clk, "setup_s": setup_s,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_null_report(args):
    """Null-space set-up at the workload's size (the reference's computeKernelCuda, ACHRCuda.cu:436-502):
    for each construction, the wall time of context creation (upload, null space, centre) and the
    quality of the basis, max|S N| and max|N^T N - I| (FP64, on the GPU)."""
    import importlib

    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    synth = importlib.import_module("achr_gb300.synthetic")
    spec, model, S, warm, _, _ = build_inputs(args.workload, pkg, synth, null_space=gpu_null_space_fn(pkg),
                                              warmup_form=args.warmup_form)
    St = torch.from_numpy(S).cuda()
    rows = {}
    for name, code in (("sts", pkg.NULL_SVD_STS), ("svd", pkg.NULL_SVD_S), ("fixed", pkg.NULL_FIXED)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            smp = pkg.Sampler(model, warm, null_space=code)
        except pkg.AchrError as e:
            rows[name] = {"error": str(e)}
            continue
        torch.cuda.synchronize()
        create_s = time.perf_counter() - t0
        N = torch.from_numpy(smp.null_space()).cuda()
        d = N.shape[1]
        I = torch.eye(d, dtype=torch.float64, device="cuda")
        fixed = torch.from_numpy(np.asarray(model.lb == model.ub)).cuda()
        rows[name] = {"create_s": create_s, "null_dim": d, "max_abs_SN": float((St @ N).abs().max()),
                      "max_abs_NtN_minus_I": float((N.T @ N - I).abs().max()),
                      "max_abs_N_on_fixed": float(N[fixed].abs().max()) if bool(fixed.any()) else 0.0}
        smp.close()
        del N, I
    line = {"metric": "null-space set-up", "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": "f64",
            "data": "synthetic", "config": {"workload": f"{args.workload}: {spec.n_mets}x{spec.n_rxns}, "
                                                        f"W={warm.shape[1]}, fixed reactions "
                                                        f"{int(np.sum(model.lb == model.ub))}"},
            "methods": rows}
    print(json.dumps(line), flush=True)
    return 0


def run_gemm(args):
    """The tensor-core GEMM alone on the reprojection's shape: M = 5063 (metabolites of
    the large model), K = 5120 (padded), N = --gemm CHAINS, one product and the three
    split products; CUDA-event timing over 5 calls after 2 warm-up calls."""
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    m, kpad, N = 5063, 5120, args.gemm
    g = torch.Generator(device="cuda").manual_seed(args.seed)
    A0 = torch.randn(m, kpad, device="cuda", generator=g).to(torch.bfloat16)
    A1 = (torch.randn(m, kpad, device="cuda", generator=g) * 2.0 ** -9).to(torch.bfloat16)
    B0 = torch.randn(N, kpad, device="cuda", generator=g).to(torch.bfloat16)
    B1 = (torch.randn(N, kpad, device="cuda", generator=g) * 2.0 ** -9).to(torch.bfloat16)
    C = torch.empty(m, N, device="cuda", dtype=torch.float32)
    tpeak, tpeak_kind = load_tensor_peak()
    rows = {}
    for nsplit in (1, 3):
        a1 = A1.data_ptr() if nsplit == 3 else 0
        b1 = B1.data_ptr() if nsplit == 3 else 0
        call = lambda: pkg.gemm_bf16(m, N, kpad, A0.data_ptr(), B0.data_ptr(), C.data_ptr(), kpad, kpad, N,  # noqa: E731
                                     A1=a1, B1=b1)
        for _ in range(2):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(5):
            call()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 5
        tf = 2.0 * m * N * kpad * nsplit / (ms * 1e-3) / 1e12
        rows[f"nsplit{nsplit}"] = {"ms": ms, "tflops": tf, "tensor_frac": tf / tpeak}
    line = {"metric": "TFLOP/s", "value": rows["nsplit3"]["tflops"], "unit": "TFLOP/s", "higher_is_better": True,
            "n_gpus": 1, "dtype": "bf16 x bf16 -> fp32", "data": "synthetic",
            "config": {"workload": f"tensor-core GEMM M={m} N={N} K={kpad} (reprojection shape)"},
            "peak": tpeak, "peak_source": tpeak_kind, **rows}
    print(json.dumps(line), flush=True)
    return 0


def run_cli_genome(args):
    """The drop-in command line at genome scale, as a user runs it: the 2766 x 3742 model written
    as fixed MPS, its 7484 warmup points as the reference's %f CSV (the bench's own inputs),
    `ACHRCuda model.mps warmup.csv 1 P 2000` with P = 100,000 (--chains to change), writing the
    3.7 GB File0.  Wall-clock seconds of the whole process and the CLI's own phase lines."""
    import importlib
    import tempfile

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    synth = importlib.import_module("achr_gb300.synthetic")
    spec, model, S, warm, P, T = build_inputs("genome", pkg, synth, warmup_form="percent_f")
    P = args.chains or P
    row, col, val, lb, ub = synth.make_model(spec)
    times, phases = [], []
    with tempfile.TemporaryDirectory() as tmp:
        mps, csv = Path(tmp) / "genome.mps", Path(tmp) / "genome_warmup.csv"
        synth.write_mps(mps, spec.n_mets, spec.n_rxns, row, col, val, lb, ub, name="genome")
        pkg.write_points_csv(csv, warm)
        run_dir = Path(tmp) / "run"
        run_dir.mkdir()
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            r = subprocess.run([str(pkg.cli_path()), str(mps), str(csv), "1", str(P), str(T), "--seed",
                                str(args.seed + k)], cwd=run_dir, capture_output=True, text=True)
            el = time.perf_counter() - t0
            if r.returncode != 0:
                raise SystemExit(f"ACHRCuda failed ({r.returncode}): {r.stderr[-400:]}")
            if k >= args.warmup:
                times.append(el)
                phases.append({m.group(1): float(m.group(2)) for m in
                               re.finditer(r"(Null space|Sampling) done in ([0-9.]+) seconds", r.stdout)})
        size = (run_dir / "File0").stat().st_size
        csv_bytes = csv.stat().st_size
    wall = float(np.median(times))
    line = {"metric": f"wall seconds (CLI, 1 file x {P} points x {T} steps)", "value": wall, "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "dtype": "f64",
            "data": "synthetic genome model; warmup CSV written with %f", "chain_steps_per_s": P * T / wall,
            "file0_bytes": size, "warmup_csv_bytes": csv_bytes, "runs_s": times, "phases_s": phases,
            "config": {"workload": f"genome CLI: ACHRCuda genome.mps genome_warmup.csv 1 {P} {T}"}}
    print(json.dumps(line), flush=True)
    return 0


def run_cli(args):
    """The drop-in command line on the reference's smallest published configuration: a 72 x 95
    model (the committed fixture; the paper's E. coli core has the same size), 190 warmup points
    from the LP restatement, nFiles = 1, nPoints = 1000, nSteps = 1000.  Wall-clock seconds of the
    whole process (start-up, MPS and CSV reading, null space, sampling, File0), the figure the
    reference's paper quotes (2 s on a K40 for E. coli core, 42 s for MATLAB)."""
    import tempfile

    import __graft_entry__ as ge

    pkg = ge.load_package()
    pkg.lib()
    golden = ROOT / "tests" / "golden"
    times = []
    with tempfile.TemporaryDirectory() as tmp:
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            r = subprocess.run([str(pkg.cli_path()), str(golden / "small.mps"), str(golden / "small_warmup.csv"), "1",
                                "1000", "1000", "--seed", str(args.seed + k)], cwd=tmp, capture_output=True,
                               text=True)
            el = time.perf_counter() - t0
            if r.returncode != 0:
                raise SystemExit(f"ACHRCuda failed ({r.returncode}): {r.stderr[-400:]}")
            if k >= args.warmup:
                times.append(el)
        size = (Path(tmp) / "File0").stat().st_size
    wall = float(np.median(times))
    line = {"metric": "wall seconds (CLI, 1 file x 1000 points x 1000 steps)", "value": wall, "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "dtype": "f64",
            "data": "synthetic 72 x 95 fixture (tests/golden)", "chain_steps_per_s": 1e6 / wall,
            "file0_bytes": size, "runs_s": times,
            "config": {"workload": "small CLI: ACHRCuda small.mps small_warmup.csv 1 1000 1000"}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.cli:
        return run_cli_genome(args) if args.workload == "genome" and args.chains else run_cli(args)
    if args.null_report:
        return run_null_report(args)
    if args.gemm:
        return run_gemm(args)
    if args.learned:
        return run_learned(args)
    if args.profile_case:
        return run_profile_case(args)
    if args.workload == "large" and args.impl == "gb300" and not args.ess:
        return run_large(args)
    if args.ess:
        return run_ess(args)
    if args.workload == "batch64":
        return run_batch(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
