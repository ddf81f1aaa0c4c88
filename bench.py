"""Headline benchmark: nonnegative CPD-ALS time to target fit on one GB300.

Workload (the 1000^3 configuration): 3-way dense tensor 1000 x 1000 x 1000, rank R=32,
ground-truth factors i.i.d. U[0,1] with column norms equalised (seed 2), 30 dB Gaussian
noise, initial factors U[0,1] (seed 3), nonnegativity on every mode, reference defaults
otherwise (Nesterov delta 1e-2, acceleration and normalisation on).  Synthetic data of
that shape stands in for user data.

A step is one full solve to the target: relative fit error <= noise floor + 1e-3, where the
noise floor ||noise||/||X|| (computed in FP64 when the data is generated) is the error the
FP64 least-squares optimum reaches up to O(R*sum(I)/prod(I)) = 1e-4 of overfit, so the
target is "within 1e-3 of the FP64 oracle's converged fit".

  value    BF16 tensor storage + tcgen05 MTTKRP until the fit reaches the target, then the
           final factors' fit measured on the FP32 copy (one FP32 MTTKRP, Gram form); tensor
           already resident in HBM (seconds per solve, lower is better)
  plain    the same solve with FP32 storage and CUDA-core MTTKRP (reported beside it)
  e2e      the one-call C ABI (ptg_cpd) from a pinned host FP64 buffer: host->device copy,
           BF16 and FP32 conversion, solve, factor download, all inside the timed region
  roofline MTTKRP launches timed live with CUDA events on their stream inside the timed
           region; algorithmic bytes = prod(I)*2 + sum_{k != n} I_k*R*4 + I_n*R*4
  cpu_baseline  the FP64 OpenMP restatement of the reference's CpdOpenMP (oracle/cpd_omp.c)
           on the host cores, one full-size ALS sweep timed and scaled by the sweeps the FP64
           algorithm needs (the FP32 plain form tracks the FP64 trajectory sweep by sweep)

Inputs (2 GB BF16, 4 GB FP32) are far larger than the 129 MB L2, so no flush is needed
between steps.  ``--impl reference`` times the CPU restatement alone.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = [1000, 1000, 1000]
RANK = 32
SEED, INIT_SEED, SNR_DB = 2, 3, 30.0
METRIC = "time to rel. fit err <= FP64-oracle fit + 1e-3 (BF16 tcgen05 MTTKRP, fit verified on FP32 data), 1000^3 R=32 nonneg CPD-ALS"
# Sweeps the FP64 ALS needs to reach the target on this workload (measured with the FP32
# plain form, whose per-sweep relative error follows the FP64 oracle within 1e-4).
SWEEPS_TO_TARGET_FP64 = None   # filled from the plain-form run when available


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", os.environ.get("LOCAL_RANK", "0")],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sweep_seconds(X_host_flat, dims, R, init, threads, sweeps=1):
    """One (or more) full-size FP64 ALS sweeps of the OpenMP restatement; seconds per sweep."""
    from oracle import omp
    t = time.perf_counter()
    fs, st, tr = omp.cpd_als(X_host_flat, dims, R, init, max_iter=sweeps, threshold_error=0.0,
                             nthreads=threads)
    return (time.perf_counter() - t) / sweeps, st


def run_reference(args):
    """CPU restatement of the reference (oracle/cpd_omp.c, FP64, all host threads)."""
    ws, rank = _dist()
    if rank != 0:
        return
    import numpy as np
    import torch
    ge = __import__("__graft_entry__")
    pkg = ge.load_package()
    from partensor_toolbox_gb300 import datagen as dg
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    p = dg.make_cpd_problem(DIMS, RANK, seed=SEED, init_seed=INIT_SEED, snr_db=SNR_DB,
                            equalize_columns=True, device=dev)
    Xh = p.X.cpu().numpy()
    init = [f.cpu().numpy() for f in p.init_factors]
    del p
    threads = os.cpu_count() or 1
    sweeps = args.sweeps_to_target
    times = []
    for _ in range(max(0, args.warmup_ref)):
        cpu_sweep_seconds(Xh, DIMS, RANK, init, threads)
    for _ in range(args.steps):
        s, _ = cpu_sweep_seconds(Xh, DIMS, RANK, init, threads)
        times.append(s)
    per_sweep = statistics.mean(times)
    value = per_sweep * sweeps
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_sweep * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "cpd_als 1000x1000x1000 R=32 30dB nonneg",
                                            "rank": RANK, "dims": DIMS, "l2": "inputs > L2"},
            "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                             "sample": f"1 full-size FP64 ALS sweep per step (OpenMP restatement of "
                                       f"CpdOpenMP, oracle/cpd_omp.c), x {sweeps} sweeps to target"},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    ge = __import__("__graft_entry__")
    pkg = ge.load_package()
    from partensor_toolbox_gb300 import datagen as dg
    dims, R = (args.dims or DIMS) if not args.small else [200, 200, 200], RANK
    p = dg.make_cpd_problem(dims, R, seed=SEED, init_seed=INIT_SEED, snr_db=SNR_DB, equalize_columns=True,
                            device="cuda")
    target = p.noise_rel + 1e-3
    init = [f.cpu().numpy() for f in p.init_factors]
    ctx = pkg.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    Xb = pkg.Tensor(ctx, (p.X.data_ptr(), dims), precision="bf16")
    Xf = pkg.Tensor(ctx, (p.X.data_ptr(), dims), precision="f32")
    max_iter = args.max_iter

    def solve(form):
        if form == "bf16":
            o = pkg.Options(order=3, max_iter=max_iter, threshold_error=target, precision="bf16",
                            verify_fp32=True)
            return pkg.cpd_resident(ctx, Xb, R, o, init, refine=Xf)
        o = pkg.Options(order=3, max_iter=max_iter, threshold_error=target)
        return pkg.cpd_resident(ctx, Xf, R, o, init)

    def timed(form, k, stats=False):
        sts = []
        torch.cuda.synchronize()
        _barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if stats:
            ctx.enable_stats(True)
            ctx.reset_stats()
        e0.record(stream)
        for _ in range(k):
            sts.append(solve(form))
        e1.record(stream)
        torch.cuda.synchronize()
        _barrier(ws)
        st_k = ctx.stats() if stats else None
        if stats:
            ctx.enable_stats(False)
        ms = e0.elapsed_time(e1) / k
        return ms, sts, st_k

    for _ in range(args.warmup):
        solve("bf16")
    solve("f32")
    clk = ClockSampler()
    clk.start()
    ms_b, st_b, kst = timed("bf16", args.steps, stats=True)
    clocks = clk.stop()
    ms_f, st_f, _ = timed("f32", max(1, args.steps_plain))
    ms_b = _max_over_ranks(ms_b, ws)
    ms_f = _max_over_ranks(ms_f, ws)

    # roofline of the dominant kernel (MTTKRP, tensor-core form)
    peak, peak_kind = _peaks()
    launches = max(1, kst["tc_launches"])
    per_launch_ms = kst["tc_ms"] / launches
    bytes_per_launch = kst["tc_bytes"] / launches
    achieved = bytes_per_launch / (per_launch_ms * 1e-3) / 1e9
    # DRAM bytes per launch from the ncu capture of the same kernel at 640^3 (mode 1):
    # read 530.58 MB + write 3.66 MB, scaled by the tensor entries of this workload
    traffic = (530.58e6 + 3.66e6) / 640 ** 3 * float(np.prod(dims))

    # end-to-end through the one-call C ABI with a pinned host FP64 buffer
    e2e = None
    if not args.no_e2e:
        host = torch.empty(p.X.numel(), dtype=torch.float64, pin_memory=True)
        host.copy_(p.X)
        hnp = host.numpy()
        o = pkg.Options(order=3, max_iter=max_iter, threshold_error=target, precision="bf16", verify_fp32=True)
        pkg.cpd(hnp, R, o, init, dims=dims, ctx=ctx)   # warm-up
        ts = []
        for _ in range(max(1, args.steps_e2e)):
            torch.cuda.synchronize()
            t = time.perf_counter()
            st_e = pkg.cpd(hnp, R, o, init, dims=dims, ctx=ctx)
            ts.append(time.perf_counter() - t)
        # the host side is shared with other jobs on this machine: its memory and host-to-GPU
        # link vary from call to call, so the spread of the calls is reported beside the mean
        e2e = {"value": _max_over_ranks(statistics.mean(ts), ws), "unit": "s",
               "h2d_bytes_per_step": int(hnp.nbytes + sum(f.nbytes for f in init)),
               "d2h_bytes_per_step": int(sum(f.nbytes for f in st_e.factors)),
               "rel_err": st_e.rel_costFunction, "min": min(ts), "median": statistics.median(ts),
               "calls_s": [round(x, 5) for x in ts]}
        del host

    sweeps_plain = st_f[-1].ao_iter
    cpu = None
    if rank == 0 and not args.no_cpu:
        Xh = p.X.cpu().numpy()
        threads = os.cpu_count() or 1
        s_sweep, _ = cpu_sweep_seconds(Xh, dims, R, init, threads)
        cpu = {"value": s_sweep * sweeps_plain, "unit": "s", "cores": threads, "kind": "port",
               "sample": f"1 full-size FP64 ALS sweep of the OpenMP restatement of CpdOpenMP "
                         f"(oracle/cpd_omp.c) = {s_sweep:.2f} s, x {sweeps_plain} sweeps to target "
                         f"(the FP32 plain form's count)"}
        del Xh

    last_b, last_f = st_b[-1], st_f[-1]
    line = {
        "metric": METRIC, "value": ms_b / 1e3, "unit": "s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_b, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded U[0,1] factors, 30 dB Gaussian noise)",
        "config": {"workload": f"cpd_als {dims[0]}x{dims[1]}x{dims[2]} R={R} 30dB nonneg, to target",
                   "rank": R, "dims": dims, "target_rel": target, "noise_floor_rel": p.noise_rel,
                   "l2": "inputs (2 GB BF16 / 4 GB FP32) > 129 MB L2, no flush",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "converged": bool(last_b.rel_costFunction <= target),
        "fit_measured_on": "FP32 copy of the tensor (final factors)",
        "final_rel_err": last_b.rel_costFunction,
        "sweeps": last_b.ao_iter, "refine_sweeps": last_b.refine_sweeps_done,
        "nesterov_iters_total": last_b.nesterov_iters_total,
        "plain_fp32": {"value": ms_f / 1e3, "unit": "s", "sweeps": sweeps_plain,
                       "final_rel_err": last_f.rel_costFunction,
                       "converged": bool(last_f.rel_costFunction <= target)},
        "speedup_vs_plain_fp32": (ms_f / ms_b) if ms_b > 0 else None,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "mttkrp_tc_kernel + tc_reduce_kernel (tcgen05, BF16 storage)",
                     "launches": kst["tc_launches"], "ms_per_launch": per_launch_ms,
                     "bytes_per_launch": bytes_per_launch,
                     "traffic_source": "ncu capture at 640^3 scaled by entries (profiles/)"},
        "gpu_launches": kst["launches"],
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    Xb.close()
    Xf.close()
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


BATCH_N, BATCH_SEED = 256, 4
BATCH_METRIC = ("instances/s, 256 uneven fMRI-like nonneg CPDs (dims U[32,128]xU[100,400]xU[16,64], "
                "R in {8,12,16,24}, 15 dB) each to its FP64-oracle fit + 1e-3")


def _batch_problems():
    from partensor_toolbox_gb300 import datagen as dg
    batch = dg.make_fmri_batch(BATCH_N, seed=BATCH_SEED)
    return [(b.X, b.rank, b.init_factors, b.noise_rel + 1e-3) for b in batch]


def _batch_cpu(probs, sample, threads):
    """The FP64 OpenMP restatement on the first `sample` instances, each to its target."""
    from oracle import omp
    t = time.perf_counter()
    iters = []
    for X, R, init, thr in probs[:sample]:
        _, st, _ = omp.cpd_als(X.reshape(-1, order="F"), list(X.shape), R, init, threshold_error=thr,
                               max_iter=200, nthreads=threads)
        iters.append(st.ao_iter)
    return time.perf_counter() - t, iters


def run_batch_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return
    ge = __import__("__graft_entry__")
    ge.load_package()
    probs = _batch_problems()
    threads = os.cpu_count() or 1
    sample = args.batch_sample
    for _ in range(max(0, args.warmup_ref)):
        _batch_cpu(probs, sample, threads)
    ts = [_batch_cpu(probs, sample, threads)[0] for _ in range(args.steps)]
    value = sample / statistics.mean(ts)
    line = {"impl": "reference", "metric": BATCH_METRIC, "value": value, "unit": "instances/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(ts) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded fMRI-like batch, seed 4)",
            "config": {"workload": "cpd_batched fmri-like 256 instances", "instances": BATCH_N},
            "cpu_baseline": {"value": value, "unit": "instances/s", "cores": threads, "kind": "port",
                             "sample": f"first {sample} of the 256 instances per step, FP64 OpenMP "
                                       f"restatement of CpdOpenMP (oracle/cpd_omp.c), each to its target"},
            "e2e": {"value": value, "unit": "instances/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batch_ours(args):
    import numpy as np
    import torch
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ge = __import__("__graft_entry__")
    pkg = ge.load_package()
    probs = _batch_problems()
    ctx = pkg.Context(local)
    opts = pkg.Options(order=3, max_iter=200)
    for _ in range(args.warmup):
        pkg.cpd_batched(probs, opts, ctx=ctx)
    ctx.enable_stats(True)
    clk = ClockSampler()
    clk.start()
    walls, solves, conv = [], [], []
    launches = 0
    for _ in range(args.steps):
        ctx.reset_stats()
        torch.cuda.synchronize()
        t = time.perf_counter()
        sts, secs = pkg.cpd_batched(probs, opts, ctx=ctx)
        walls.append(time.perf_counter() - t)
        solves.append(float(secs.max()))
        conv.append(secs)
        kst = ctx.stats()
        launches += kst["launches"]
    clocks = clk.stop()
    ctx.enable_stats(False)
    secs = np.concatenate(conv)
    hit = sum(st.rel_costFunction <= p[3] for st, p in zip(sts, probs))
    solve_s = _max_over_ranks(statistics.mean(solves), ws)
    wall_s = _max_over_ranks(statistics.mean(walls), ws)
    peak, peak_kind = _peaks()
    ach = kst["batch_pass_bytes"] / (kst["batch_pass_ms"] * 1e-3) / 1e9 if kst["batch_pass_ms"] > 0 else None
    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        tcpu, it_cpu = _batch_cpu(probs, args.batch_sample, threads)
        cpu = {"value": args.batch_sample / tcpu, "unit": "instances/s", "cores": threads, "kind": "port",
               "sample": f"first {args.batch_sample} instances, FP64 OpenMP restatement of CpdOpenMP "
                         f"(oracle/cpd_omp.c), each to its target ({sum(it_cpu)} sweeps)"}
    h2d = int(sum(p[0].nbytes + sum(f.nbytes for f in p[2]) for p in probs))
    d2h = int(sum(sum(f.nbytes for f in st.factors) for st in sts))
    line = {
        "metric": BATCH_METRIC, "value": ws * BATCH_N / solve_s, "unit": "instances/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": solve_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded fMRI-like batch: sparse spatial maps, smooth time courses, 15 dB)",
        "config": {"workload": "cpd_batched fmri-like 256 instances", "instances": BATCH_N, "seed": BATCH_SEED,
                   "l2": "824 MB of FP32 tensors > 129 MB L2, no flush",
                   "timing": "ALS loop with every tensor resident (host clock around the graph-replayed loop)"},
        "p50_s": float(np.percentile(secs, 50)), "p99_s": float(np.percentile(secs, 99)),
        "instances_converged": int(hit), "sweeps_mean": float(np.mean([st.ao_iter for st in sts])),
        "sweeps_max": int(max(st.ao_iter for st in sts)),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": (ach / peak) if ach else None, "traffic": None, "peak_kind": peak_kind,
                     "kernel": "mttkrp_simt_batched_kernel + batched_reduce_kernel (one pass: every mode "
                               "of every instance)",
                     "launches": kst["batch_pass_launches"], "ms_per_pass": kst["batch_pass_ms"],
                     "bytes_per_pass": kst["batch_pass_bytes"]},
        "gpu_launches": launches,
        "clocks": clocks,
        "e2e": {"value": ws * BATCH_N / wall_s, "unit": "instances/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def run_dimtree(args):
    """160^4, R=64, collinear factors (cosine 0.6, seed 3), 25 dB: cpdDimTree in FP32 to the
    target (noise floor + 1e-3) is the value; beside it the direct (non-tree) FP32 solve, the
    FP32 tree with the learned warm start and the tree on BF16 tcgen05 storage with the fit
    verified on FP32."""
    import numpy as np
    import torch
    ws, rank = _dist()
    torch.cuda.set_device(0)
    ge = __import__("__graft_entry__")
    pkg = ge.load_package()
    from partensor_toolbox_gb300 import datagen as dg
    dims, R = [160, 160, 160, 160], 64
    p = dg.make_cpd_problem(dims, R, seed=3, init_seed=4, snr_db=25.0, collinearity=0.6, device="cuda")
    target = p.noise_rel + 1e-3
    init = [f.cpu().numpy() for f in p.init_factors]
    ctx = pkg.Context(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    Xb = pkg.Tensor(ctx, (p.X.data_ptr(), dims), precision="bf16")
    Xf = pkg.Tensor(ctx, (p.X.data_ptr(), dims), precision="f32")
    mi = args.max_iter

    def run(form, dimtree=True, warm=False):
        kw = dict(order=4, max_iter=mi, threshold_error=target)
        if form == "bf16":
            kw.update(precision="bf16", verify_fp32=True)
        if warm:
            kw.update(warm_start=True, warm_model=pkg.WarmStartModel(ctx, R, seed=7), warm_log_sweeps=5,
                      warm_train_steps=300)
        o = pkg.Options(**kw)
        X = Xb if form == "bf16" else Xf
        torch.cuda.synchronize()
        t = time.perf_counter()
        st = pkg.cpd_resident(ctx, X, R, o, init, refine=Xf if form == "bf16" else None, dimtree=dimtree)
        torch.cuda.synchronize()
        return time.perf_counter() - t, st

    for _ in range(max(1, args.warmup)):
        run("f32")
    res = {}
    ctx.enable_stats(True)
    clk = ClockSampler()
    clk.start()
    for name, form, dt, warm in [("dimtree_f32", "f32", True, False), ("direct_f32", "f32", False, False),
                                 ("dimtree_f32_warm", "f32", True, True), ("dimtree_bf16", "bf16", True, False)]:
        ts, st = [], None
        ctx.reset_stats()
        for _ in range(max(1, args.steps if name == "dimtree_f32" else 1)):
            t, st = run(form, dt, warm)
            ts.append(t)
        kst = ctx.stats()
        res[name] = {"seconds": statistics.mean(ts), "sweeps": st.ao_iter, "final_rel_err": st.rel_costFunction,
                     "converged": bool(st.rel_costFunction <= target),
                     "nesterov_iters_total": st.nesterov_iters_total,
                     "nesterov_iters_after_sweep5": int(sum(sum(t["nesterov_iters"]) for t in st.trace[5:])),
                     "gpu_launches": kst["launches"] // max(1, len(ts)),
                     "ms_per_sweep": 1e3 * statistics.mean(ts) / max(1, st.ao_iter),
                     "mttkrp_ms_per_sweep": kst["mttkrp_ms"] / max(1, len(ts)) / max(1, st.ao_iter)}
        if name == "dimtree_f32":
            tc = kst
    clocks = clk.stop()
    ach = tc["mttkrp_bytes"] / (tc["mttkrp_ms"] * 1e-3) / 1e9 if tc["mttkrp_ms"] > 0 else None
    cpu = None
    if not args.no_cpu:
        Xh = p.X.cpu().numpy()
        threads = os.cpu_count() or 1
        s_sweep, _ = cpu_sweep_seconds(Xh, dims, R, init, threads)
        sw = res["dimtree_f32"]["sweeps"]
        cpu = {"value": s_sweep * sw, "unit": "s", "cores": threads, "kind": "port",
               "sample": f"1 full-size FP64 ALS sweep of the OpenMP restatement of CpdOpenMP (oracle/cpd_omp.c, "
                         f"direct MTTKRP, no dimension tree) = {s_sweep:.2f} s, x {sw} sweeps"}
        del Xh
    peak, peak_kind = _peaks()
    line = {"metric": "time to rel. fit err <= noise floor + 1e-3, 160^4 R=64 collinear nonneg cpdDimTree (FP32)",
            "value": res["dimtree_f32"]["seconds"], "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": False, "dtype": "f32",
            "data": "synthetic (U[0,1] factors with a shared component, cosine 0.6, seed 3; 25 dB)",
            "config": {"workload": "cpdDimTree 160x160x160x160 R=64", "target_rel": target,
                       "noise_floor_rel": p.noise_rel, "max_iter": mi},
            "runs": res, "cpu_baseline": cpu,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": (ach / peak) if ach else None, "peak_kind": peak_kind,
                         "kernel": "MTTKRP contractions of the FP32 dimension tree (node contractions, leaves, "
                                   "acceleration cost), summed event time",
                         "launches": tc["mttkrp_launches"]},
            "clocks": clocks}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_gtc(args):
    """50000 x 50000 x 5000, 200 M observed entries sampled uniformly without replacement
    (seed 5), values from a rank-32 U[0,1] model with 10% relative Gaussian noise; 1% held out.
    Stochastic GTC (c = 0.01, lambda = 1e-3, R = 32) on device-resident int32 COO + FP32
    values; reports observed entries/s and the held-out RMSE."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    ge = __import__("__graft_entry__")
    pkg = ge.load_package()
    dims, R, total_nnz = [50000, 50000, 5000], 32, int(args.gtc_nnz)
    g = torch.Generator(device="cuda").manual_seed(5)
    cells = dims[0] * dims[1] * dims[2]
    flat = torch.unique(torch.randint(0, cells, (int(total_nnz * 1.001) + 1024,), generator=g, device="cuda"))
    flat = flat[torch.randperm(flat.numel(), generator=g, device="cuda")][:total_nnz]
    A = [torch.rand(I, R, generator=g, device="cuda") for I in dims]
    idx = torch.empty(3, total_nnz, dtype=torch.int32, device="cuda")
    vals = torch.empty(total_nnz, dtype=torch.float32, device="cuda")
    clean = torch.empty(total_nnz, dtype=torch.float32, device="cuda")
    for s in range(0, total_nnz, 1 << 24):
        f = flat[s:s + (1 << 24)]
        i0, i1, i2 = f % dims[0], (f // dims[0]) % dims[1], f // (dims[0] * dims[1])
        idx[0, s:s + f.numel()], idx[1, s:s + f.numel()], idx[2, s:s + f.numel()] = i0, i1, i2
        v = (A[0][i0] * A[1][i1] * A[2][i2]).sum(1)
        clean[s:s + f.numel()] = v
        vals[s:s + f.numel()] = v * (1 + 0.1 * torch.randn(v.shape, generator=g, device="cuda"))
    del flat
    n_hold = total_nnz // 100
    n_train = total_nnz - n_hold
    idx_tr = idx[:, :n_train].contiguous()
    vals_tr = vals[:n_train].contiguous()
    idx_ho, vals_ho, clean_ho = idx[:, n_train:], vals[n_train:], clean[n_train:]
    ctx = pkg.Context(0)
    init = [np.random.default_rng(k).random((I, R)) for k, I in enumerate(dims)]

    def rmse(factors):
        F = [torch.tensor(np.asarray(f), dtype=torch.float32, device="cuda") for f in factors]
        pred = (F[0][idx_ho[0].long()] * F[1][idx_ho[1].long()] * F[2][idx_ho[2].long()]).sum(1)
        return float(torch.sqrt(torch.mean((pred - vals_ho) ** 2)))

    out = {}
    for name, stoch, it in [("stochastic", True, args.gtc_epochs), ("full", False, args.gtc_full_iters)]:
        o = pkg.SparseOptions(order=3, rank=R, tnsDims=dims, max_iter=it, lambdas=[1e-3] * 3,
                              c_stochastic_perc=args.gtc_c, factorsInit=init, threshold_error=0.0)
        pkg.gtc_device(idx_tr.data_ptr(), vals_tr.data_ptr(), n_train,
                       dataclasses_replace(o, max_iter=1), stochastic=stoch, ctx=ctx)   # warm-up
        torch.cuda.synchronize()
        t = time.perf_counter()
        st = pkg.gtc_device(idx_tr.data_ptr(), vals_tr.data_ptr(), n_train, o, stochastic=stoch, ctx=ctx)
        torch.cuda.synchronize()
        el = time.perf_counter() - t
        passes = st.epochs if stoch else st.ao_iter
        out[name] = {"seconds": el, "seconds_setup": st.seconds_setup, "ao_iter": st.ao_iter, "epochs": st.epochs,
                     "observed_entries_per_s": n_train * max(1, passes) / el,
                     "rel_cost": st.rel_costFunction, "heldout_rmse": rmse(st.factors)}
    floor = float(torch.sqrt(torch.mean((clean_ho - vals_ho) ** 2)))
    line = {"metric": f"observed entries/s, stochastic GTC 50000x50000x5000, {total_nnz / 1e6:g}M entries, R=32, "
                      f"c={args.gtc_c:g}",
            "value": out["stochastic"]["observed_entries_per_s"], "unit": "entries/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (uniform sample, rank-32 model, 10% noise)",
            "config": {"workload": "gtc_stochastic 50000x50000x5000", "nnz_train": n_train, "nnz_heldout": n_hold,
                       "rank": R, "lambda": 1e-3, "c_stochastic_perc": args.gtc_c},
            "runs": out, "heldout_rmse_noise_floor": floor}
    print(json.dumps(line), flush=True)
    ctx.close()


def dataclasses_replace(o, **kw):
    import dataclasses
    return dataclasses.replace(o, **kw)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--steps-plain", type=int, default=2)
    ap.add_argument("--steps-e2e", type=int, default=5)
    ap.add_argument("--max-iter", type=int, default=200)
    ap.add_argument("--small", action="store_true", help="200^3 smoke configuration")
    ap.add_argument("--dims", type=int, nargs=3, default=None, help="override the tensor shape (profiling)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--warmup-ref", type=int, default=0)
    ap.add_argument("--sweeps-to-target", type=int, default=20)
    ap.add_argument("--workload", default="cpd-1000", choices=["cpd-1000", "fmri-batch", "dimtree-160", "gtc-sparse"],
                    help="cpd-1000: the headline 1000^3 solve; fmri-batch: 256 small CPDs in one call; "
                         "dimtree-160: 160^4 R=64 cpdDimTree; gtc-sparse: 200M-entry stochastic completion")
    ap.add_argument("--gtc-nnz", type=float, default=200e6)
    ap.add_argument("--gtc-epochs", type=int, default=2, help="stochastic GTC epochs (its max_iter)")
    ap.add_argument("--gtc-full-iters", type=int, default=2)
    ap.add_argument("--gtc-c", type=float, default=0.01, help="sampled fraction of each row per inner step")
    ap.add_argument("--batch-sample", type=int, default=32, help="instances the CPU baseline solves")
    args = ap.parse_args()
    if args.workload == "fmri-batch":
        run_batch_reference(args) if args.impl == "reference" else run_batch_ours(args)
    elif args.workload == "dimtree-160":
        run_dimtree(args)
    elif args.workload == "gtc-sparse":
        run_gtc(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
