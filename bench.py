#!/usr/bin/env python3
"""Headline benchmark: 200-nt MEA folds/s on GB300.

Workload (one step): 10,000 sequences x 200 nt, bases i.i.d. uniform ACGU
(np.random.default_rng(0).integers(0, 4, (10000, 200))), forced-unpaired mask
Bernoulli(0.1) (np.random.default_rng(1).random((10000, 200)) < 0.1), full MEA
fold per sequence: FP32 inside, outside, posterior and the gamma = 6 decode
with traceback (bitwise the reference's float32 engine).

  value  : folds/s of the batched (length-bucketed) plan with inputs resident in
           HBM, CUDA events around each step on the launch stream, L2 flushed
           (256 MiB write) between steps, max over ranks.
  plain  : the same with the plain one-sequence-per-CTA launch shape.
  e2e    : folds/s through the public API (contrafold_gpu_gb300.gpu.mea_batch:
           Python strings in, dot-brackets out; host->device and device->host
           copies inside the timed region).
  roofline : the dominant kernel's algorithmic FP32 operations (guarded
           semiring updates counted exactly on a sample of the workload by the
           oracle, scaled to the batch) / its CUDA-event time, against the FP32
           issue peak (SMs x 128 lanes x max SM clock).
  cpu_baseline : the oracle (C restatement of the reference's CPU engine) on
           all host cores over a bounded sample of the same workload.

`--impl reference` times the reference's CPU engine (the oracle port, all host
threads) on the same workload, one bounded sample per step.

Multi-GPU (torchrun): replicas, each rank folds its own 10,000-sequence batch
(weak scaling); no collective on the data path.
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

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "200-nt MEA folds/s, batched vs plain on 1 GB300 at logZ≤5e-4; served p50/p99 ms"
UNIT = "folds/s"


def workload(n: int, L: int, p_mask: float = 0.1):
    from contrafold_gpu_gb300 import workloads
    return workloads.mea_200(n, L, p_mask)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"cf_bench_clocks_dev{device}_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    try:
        with open(os.path.join(REPO, "profiles", "ncu_traffic.json")) as fh:
            return json.load(fh)
    except Exception:
        return None


# --------------------------------------------------------------------------- CPU baseline leg
def cpu_baseline_leg(seq_bytes, mask, gpu_structs, budget_s: float = 12.0):
    """Oracle (C restatement of the reference CPU engine) on all host cores over a
    bounded sample of the workload; also the exact guarded-update counts of a
    sample for the roofline and a structure cross-check of the GPU output."""
    import contrafold_gpu_gb300 as cg
    from oracle import oracle as O
    O.build()
    P = cg.load()
    cores = os.cpu_count() or 1
    n, L = seq_bytes.shape
    seqs = [bytes(r).decode() for r in seq_bytes]
    masks = [m for m in mask]
    # exact op counts on 32 sequences of the workload
    cnt = np.zeros(8, np.float64)
    ns = min(32, n)
    for b in range(ns):
        cnt += O.count_mea_ops(seqs[b], P, masks[b], 6.0)
    counts_per_fold = cnt / ns
    # timed sample: grow in chunks of 4*cores until the budget is spent
    done, t_total, match = 0, 0.0, True
    chunk = max(16, 4 * cores)
    while done < n and t_total < budget_s:
        sl = slice(done, min(n, done + chunk))
        t0 = time.perf_counter()
        out = O.batch(O.JOB_MEA, seqs[sl], P, masks[sl], 6.0, threads=cores)
        t_total += time.perf_counter() - t0
        if gpu_structs is not None:
            match &= out == gpu_structs[sl]
        done = sl.stop
    return {"value": done / t_total, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {done} sequences of the workload (MEA gamma=6, 200 nt, 10% mask), "
                      f"{cores} threads, {t_total:.1f} s",
            "structures_match_gpu": bool(match)}, counts_per_fold


# --------------------------------------------------------------------------- reference arm
def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import contrafold_gpu_gb300 as cg
    from oracle import oracle as O
    O.build()
    P = cg.load()
    cores = os.cpu_count() or 1
    seq_bytes, mask = workload(args.n, args.L)
    per = max(32, 4 * cores)
    seqs = [bytes(r).decode() for r in seq_bytes[: per * (args.steps + args.warmup)]]
    masks = list(mask[: per * (args.steps + args.warmup)])
    for w in range(args.warmup):
        O.batch(O.JOB_MEA, seqs[w * per:(w + 1) * per], P, masks[w * per:(w + 1) * per], 6.0, threads=cores)
    t = 0.0
    for k in range(args.steps):
        o = (args.warmup + k) * per
        t0 = time.perf_counter()
        O.batch(O.JOB_MEA, seqs[o:o + per], P, masks[o:o + per], 6.0, threads=cores)
        t += time.perf_counter() - t0
    v = per * args.steps / t
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(args), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per} sequences of the workload per step, {cores} threads "
                                       f"(C restatement of gpu_contrafold/cpu.py posterior + mea_decode)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def config_dict(args):
    return {"workload": f"MEA fold (inside+outside+posterior+gamma=6 decode), {args.n} x {args.L} nt i.i.d. ACGU, "
                        f"Bernoulli(0.1) forced-unpaired mask",
            "n_seqs": args.n, "seq_len": args.L, "gamma": 6.0, "mask_p": 0.1,
            "l2": "flushed between steps (256 MiB write); arena per step exceeds L2",
            "parallelism": f"replicas x{args.gpus}"}


# --------------------------------------------------------------------------- our arm
def our_arm(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import contrafold_gpu_gb300 as cg
    from contrafold_gpu_gb300 import build as cbuild
    from contrafold_gpu_gb300.engine import CF_JOB_MEA, CF_JOB_LOGZ, CF_JOB_LOGZ64, Engine, Plan
    if rank == 0:
        cbuild.build()
    if dist is not None:
        dist.barrier()
    P = cg.load()
    n, L = args.n, args.L
    seq_bytes, mask = workload(n, L)
    offsets = np.arange(n + 1, dtype=np.int64) * L
    dev = torch.device("cuda", local)
    d_seqs = torch.from_numpy(seq_bytes.reshape(-1).copy()).to(dev)
    d_mask = torch.from_numpy(mask.reshape(-1).copy()).to(dev)
    d_out = torch.empty(n * L, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # a dedicated stream: its handle is what the plan launches on and what the
    # CUDA events below are recorded on (the legacy default stream's handle is 0)
    stream = torch.cuda.Stream(dev)

    def sync_all():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    def run_mode(mode, timing=True, schedule="auto"):
        eng = Engine(P, device=local, mode=mode)
        if mode == "batched":
            eng.set_schedule(schedule)
        plan = Plan(eng, CF_JOB_MEA, offsets)
        plan.set_timing(timing)
        for _ in range(args.warmup):
            plan.run(d_seqs.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), 6.0, stream.cuda_stream)
        plan.status()
        step_ms, phase = [], np.zeros(4)
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            sync_all()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.run(d_seqs.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), 6.0, stream.cuda_stream)
            e1.record(stream)
            sync_all()
            step_ms.append(e0.elapsed_time(e1))
            if timing:
                phase += plan.phase_ms()
        plan.status()
        res = {"step_ms": step_ms, "phase_ms": phase / args.steps, "launches": plan.launches * args.steps,
               "group": plan.group, "arena_bytes": plan.arena_bytes, "schedule": plan.schedule}
        plan.close()
        eng.close()
        return res

    # plain launch shape first (the reference's one-sequence-per-block kernels),
    # the length-grouped per-sequence kernels, then the batched path under the
    # clock sampler
    plain = run_mode("plain")
    grouped = run_mode("batched", schedule="group")
    # the batched plan runs untimed per phase: a grouped MEA plan is then one
    # fused launch per step (per-phase timing would split it into four)
    with ClockSampler(local) as clk:
        batched = run_mode("batched", timing=False)
    clocks = clk.summary()
    structs = d_out.cpu().numpy().reshape(n, L).tobytes().decode("ascii")
    gpu_structs = [structs[b * L:(b + 1) * L] for b in range(n)]

    def agg(total_ms):
        t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    t_b = agg(sum(batched["step_ms"]))
    t_p = agg(sum(plain["step_ms"]))
    t_g = agg(sum(grouped["step_ms"]))
    value = n * args.steps * world / (t_b / 1000.0)
    plain_value = n * args.steps * world / (t_p / 1000.0)

    # e2e through the public API (strings in, structures out)
    seq_strs = [bytes(r).decode() for r in seq_bytes]
    masks = list(mask)
    for _ in range(max(1, args.warmup // 2)):
        cg.gpu.mea_batch(seq_strs, P, 6.0, masks)
    sync_all()
    t0 = time.perf_counter()
    e2e_out = None
    for _ in range(args.steps):
        e2e_out = cg.gpu.mea_batch(seq_strs, P, 6.0, masks)
    t_e2e = agg((time.perf_counter() - t0) * 1000.0)
    e2e_value = n * args.steps * world / (t_e2e / 1000.0)
    e2e_ok = e2e_out == gpu_structs

    # logZ accuracy of the FP32 logZ path against the FP64 engine on 1,000 sequences
    m = min(1000, n)
    eng = Engine(P, device=local)
    from contrafold_gpu_gb300.engine import Batch
    Bz = Batch(seq_strs[:m], masks[:m])
    logz_err = float(np.max(np.abs(eng.logz(Bz).astype(np.float64) - eng.logz64(Bz))))
    eng.close()

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    cpu, counts = cpu_baseline_leg(seq_bytes, mask, gpu_structs)
    from oracle.oracle import OP_COST
    ph = batched["phase_ms"]
    if batched["launches"] == args.steps:
        # the batched path is one fused kernel: inside + outside + posterior + decode,
        # timed by the CUDA events around each step (one launch and a memset)
        phase_cats = {0: tuple(range(8)), 1: (), 2: (), 3: ()}
        fused = {"warp": "k_fold_warp<MEA>", "group": "k_fold_group32<MEA>", "cta": "k_fold_cta<MEA>"}
        names = {0: fused.get(batched["schedule"], batched["schedule"]), 1: "-", 2: "-", 3: "-"}
        ph = np.array([statistics.mean(batched["step_ms"]), 0.0, 0.0, 0.0])
    else:
        phase_cats = {0: (0, 1, 2), 1: (3, 4, 5), 2: (6,), 3: (7,)}
        names = {0: "k_inside32", 1: "k_outside32", 2: "k_posterior32", 3: "k_mea32"}
    dom = int(np.argmax(ph))
    ops_per_fold = {k: float(sum(counts[c] * OP_COST[c] for c in cats)) for k, cats in phase_cats.items()}
    achieved = ops_per_fold[dom] * n / (ph[dom] / 1000.0) / 1e12
    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    peak = props.multi_processor_count * 128 * sm_mhz * 1e6 / 1e12
    tr = ncu_traffic()
    traffic = None
    if tr and tr.get("kernel") == names[dom]:
        traffic = tr.get("bytes_per_launch_full")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_b / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(args),
        "plain": {"value": plain_value, "ms_per_step": t_p / args.steps,
                  "kernels": "one sequence per CTA, threads over the cells of a span, whole-window scans",
                  "phase_ms": {k: float(v) for k, v in zip(("k_plain_inside32", "k_plain_outside32",
                                                           "k_plain_posterior32", "k_plain_mea32"),
                                                           plain["phase_ms"])}},
        "grouped": {"value": n * args.steps * world / (t_g / 1000.0), "ms_per_step": t_g / args.steps,
                    "group": grouped["group"],
                    "phase_ms": {k: float(v) for k, v in zip(("k_inside32", "k_outside32", "k_posterior32", "k_mea32"),
                                                             grouped["phase_ms"])}},
        "batched_vs_plain": (t_p / t_b),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(2 * n * L + 8 * (n + 1) + 24 * n),
                "d2h_bytes_per_step": int(n * L + 4), "api": "contrafold_gpu_gb300.gpu.mea_batch",
                "matches_device_path": bool(e2e_ok)},
        "gpu_launches": int(batched["launches"]),
        "roofline": {"bound": "fp32", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_note": f"{props.multi_processor_count} SMs x 128 FP32 lanes x {sm_mhz:.0f} MHz "
                                  "(sm_max_mhz of MEASURED_PEAKS.json); the DP is a log/max semiring, "
                                  "neither HBM- nor tensor-bound",
                     "ops_per_fold": ops_per_fold[dom],
                     "phase_ms": {names[k]: float(ph[k]) for k in range(4)},
                     "hbm": None if traffic is None or not peaks.get("hbm_gbs") else {
                         "traffic_gbs": traffic / (ph[dom] / 1000.0) / 1e9,
                         "peak_gbs": float(peaks["hbm_gbs"]),
                         "frac_of_measured": traffic / (ph[dom] / 1000.0) / 1e9 / float(peaks["hbm_gbs"]),
                         "note": "ncu DRAM bytes per launch (profiles/ncu_traffic.json) over the measured launch "
                                 "time: the kernel is not HBM-bound"}},
        "ops_per_fold_total": float(sum(counts[c] * OP_COST[c] for c in range(8))),
        "logz_max_abs_err_fp32_vs_fp64": logz_err,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def decoder_arm(args):
    """The other two decoders of the 10,000 x 200 nt workload (same sequences and
    Bernoulli(0.1) masks as the headline), one JSON line each:
      bpp : base-pair posterior matrices (inside + outside + posterior, float32,
            bitwise the reference's), packed L x L float32 per sequence;
      mfe : Viterbi structures (FP64 max-plus inside + EPS first-match traceback).
    value: device-resident plan, CUDA events on the launch stream, L2 flushed
    between steps; e2e: the public batch call (bpp_batch / mfe_batch) with
    Python strings in and results out; cpu_baseline: the oracle on all host
    cores over a bounded sample."""
    import torch
    import contrafold_gpu_gb300 as cg
    from contrafold_gpu_gb300 import build as cbuild
    from contrafold_gpu_gb300.engine import CF_JOB_BPP, CF_JOB_MFE, Engine, Plan
    from oracle import oracle as O
    cbuild.build()
    P = cg.load()
    n, L = args.n, args.L
    seq_bytes, mask = workload(n, L)
    offsets = np.arange(n + 1, dtype=np.int64) * L
    dev = torch.device("cuda", 0)
    d_seqs = torch.from_numpy(seq_bytes.reshape(-1).copy()).to(dev)
    d_mask = torch.from_numpy(mask.reshape(-1).copy()).to(dev)
    bpp = args.workload == "bpp"
    d_out = (torch.empty(n * L * L, dtype=torch.float32, device=dev) if bpp
             else torch.empty(n * L, dtype=torch.uint8, device=dev))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)

    def run_mode(mode, clk=None):
        eng = Engine(P, mode=mode)
        plan = Plan(eng, CF_JOB_BPP if bpp else CF_JOB_MFE, offsets)
        for _ in range(args.warmup):
            plan.run(d_seqs.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), 6.0, stream.cuda_stream)
        plan.status()
        ms = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.run(d_seqs.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), 6.0, stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
        plan.status()
        res = {"ms": ms, "launches": plan.launches * args.steps, "schedule": plan.schedule, "group": plan.group}
        plan.close()
        eng.close()
        return res

    plain = run_mode("plain")
    with ClockSampler(0) as clk:
        batched = run_mode("batched")
    clocks = clk.summary()
    value = n * len(batched["ms"]) / (sum(batched["ms"]) / 1e3)
    seqs = [bytes(r).decode() for r in seq_bytes]
    masks = list(mask)
    # e2e through the public API
    api = cg.gpu.bpp_batch if bpp else cg.gpu.mfe_batch
    api(seqs[:256], P, masks[:256])
    t0 = time.perf_counter()
    k_e2e = max(1, min(args.steps, 3))
    for _ in range(k_e2e):
        res = api(seqs, P, masks)
    e2e = n * k_e2e / (time.perf_counter() - t0)
    # device result vs the public call (first 64 sequences)
    if bpp:
        dev_mats = d_out[: 64 * L * L].cpu().numpy().reshape(64, L, L)
        same = all(np.array_equal(dev_mats[b].astype(np.float64), res[b]) for b in range(64))
    else:
        st = d_out[: 64 * L].cpu().numpy().tobytes().decode("ascii")
        same = all(st[b * L:(b + 1) * L] == res[b] for b in range(64))
    # CPU baseline (the oracle on all host cores, bounded sample) and op counts
    O.build()
    cores = os.cpu_count() or 1
    job = O.JOB_LOGZ32 if bpp else O.JOB_MFE     # JOB_LOGZ32 runs the whole float32 posterior
    done, tt = 0, 0.0
    while done < n and tt < 12.0:
        sl = slice(done, min(n, done + 4 * cores))
        t0 = time.perf_counter()
        O.batch(job, seqs[sl], P, masks[sl], 6.0, threads=cores)
        tt += time.perf_counter() - t0
        done = sl.stop
    cnt = np.zeros(8)
    for b in range(32):
        cnt += O.count_mea_ops(seqs[b], P, masks[b], 6.0)
    cnt /= 32
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = float(measured_peaks().get("sm_max_mhz", 2070.0))
    t_step = statistics.mean(batched["ms"]) / 1e3
    if bpp:
        ops = float(sum(cnt[c] * O.OP_COST[c] for c in range(7)))
        peak = props.multi_processor_count * 128 * sm_mhz * 1e6 / 1e12
        roof = {"bound": "fp32", "unit": "TFLOP/s", "ops_per_fold": ops,
                "peak_note": f"{props.multi_processor_count} SMs x 128 FP32 lanes x {sm_mhz:.0f} MHz (derived, "
                             "sm_max_mhz of MEASURED_PEAKS.json; no measured FP32 peak there)"}
    else:
        ops = float(sum(cnt[c] * O.VITERBI_COST[c] for c in range(3)))
        peak = 1.25   # nominal GB300 FP64 rate (TFLOP/s): 2 DFMA lanes x 2 FLOP per SM per clock
        roof = {"bound": "fp64", "unit": "TFLOP/s (FP64 lane-ops counted as DFMA-equivalent FLOP: x2)",
                "ops_per_fold": ops,
                "peak_note": "nominal GB300 FP64 1.25 TFLOP/s (no measured FP64 peak); each FP64 add or compare "
                             "occupies one DFMA slot, so achieved = 2 x FP64 ops / s"}
    achieved = (ops * n / t_step / 1e12) * (1 if bpp else 2)
    roof.update({"kernel": ("k_fold_group32<BPP>" if batched["schedule"] == "group" else batched["schedule"])
                 if bpp else "k_viterbi64", "achieved": achieved, "peak": peak, "frac": achieved / peak,
                 "traffic": None})
    out_bytes = n * L * L * 4 if bpp else n * L
    line = {"metric": ("200-nt BPP folds/s" if bpp else "200-nt Viterbi (MFE) folds/s") + " on 1 GB300",
            "value": value, "unit": "folds/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(batched["ms"]), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if bpp else "f64", "data": "synthetic",
            "config": {"workload": ("BPP (inside+outside+posterior, float32 L x L per sequence)" if bpp else
                                    "Viterbi (FP64 max-plus + EPS=1e-6 first-match traceback)") +
                                   f", {n} x {L} nt i.i.d. ACGU, Bernoulli(0.1) forced-unpaired mask",
                       "n_seqs": n, "seq_len": L, "mask_p": 0.1, "schedule": batched["schedule"],
                       "group": batched["group"], "l2": "flushed between steps (256 MiB write)"},
            "plain": {"value": n * len(plain["ms"]) / (sum(plain["ms"]) / 1e3),
                      "ms_per_step": statistics.mean(plain["ms"])},
            "batched_vs_plain": statistics.mean(plain["ms"]) / statistics.mean(batched["ms"]),
            "gpu_launches": batched["launches"],
            "e2e": {"value": e2e, "unit": "folds/s", "api": "contrafold_gpu_gb300.gpu." + api.__name__,
                    "h2d_bytes_per_step": int(2 * n * L + 8 * (n + 1) + 24 * n), "d2h_bytes_per_step": out_bytes,
                    "matches_device_path": bool(same)},
            "roofline": roof,
            "cpu_baseline": {"value": done / tt, "unit": "folds/s", "cores": cores, "kind": "port",
                             "sample": f"first {done} sequences of the workload, {cores} threads, {tt:.1f} s "
                                       + ("(float32 posterior, cpu.py:583-820 restated)" if bpp else
                                          "(FP64 Viterbi + traceback, cpu.py:290-519 restated)")},
            "clocks": clocks}
    print(json.dumps(line), flush=True)
    return 0


def serving_arm(args):
    """Open-loop serving sweep: saturated throughput (every request queued at
    t = 0), then Poisson streams at fractions of it; p50 / p99 latency from the
    scheduled arrival to the result, per offered load.  Requests: log-normal
    lengths (median 150 nt, log-sd 0.6, clipped to 30-1000), 40 % logZ / 40 %
    MEA (gamma 6) / 20 % ten Boltzmann samples, 10 % carrying a Bernoulli(0.1)
    forced-unpaired mask.  A sample of results is compared with the same
    requests folded alone."""
    from contrafold_gpu_gb300 import load, serve
    from contrafold_gpu_gb300.engine import Batch, Engine
    P = load()
    out = {"metric": "serving p99 latency at 80% of saturated throughput", "unit": "ms",
           "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
           "config": {"workload": "serving: Poisson arrivals, lengths log-normal median 150 nt sigma 0.6 clipped 30-1000, "
                                  "40% logZ / 40% MEA / 20% sample x10, 10% masked",
                      "workers": args.workers, "long_workers": args.long_workers, "long_len": args.long_len,
                      "edges": args.edges, "max_batch_cost": args.max_batch_cost,
                      "max_batch_arena": args.max_batch_arena}}
    with serve.Server(P, workers=args.workers, long_workers=args.long_workers, long_len=args.long_len,
                      edges=args.edges, max_batch_cost=args.max_batch_cost,
                      max_batch_arena=args.max_batch_arena) as srv:
        warm, _ = serve.mixed_workload(2000, rate=1e9, seed=99)
        srv.replay(warm, np.zeros(len(warm)), keep_results=False)
        n_sat = args.serve_n
        reqs, _ = serve.mixed_workload(n_sat, rate=1e9, seed=100)
        with ClockSampler(0) as clk:
            rep = srv.replay(reqs, np.zeros(n_sat), keep_results=False)
            sat = n_sat / (rep.latency_ms.max() / 1e3)
            points = []
            check_frac = min(args.serve_fracs, key=lambda f: abs(f - 0.8))
            for frac in args.serve_fracs:
                rate = frac * sat
                n = max(500, int(rate * args.serve_seconds))
                reqs, t = serve.mixed_workload(n, rate=rate, seed=int(frac * 1000))
                st0 = srv.stats()
                rep = srv.replay(reqs, t, keep_results=(frac == check_frac))
                st1 = srv.stats()
                lat = rep.latency_ms
                pt = {"offered_frac": frac, "offered_rps": round(rate, 1),
                      "achieved_rps": round(n / float(np.max(t + lat / 1e3)), 1),
                      "p50_ms": round(float(np.percentile(lat, 50)), 3),
                      "p99_ms": round(float(np.percentile(lat, 99)), 3),
                      "max_ms": round(float(lat.max()), 3),
                      "mean_batch": round((st1["done"] - st0["done"]) / max(1, st1["batches"] - st0["batches"]), 1),
                      "errors": int(np.count_nonzero(rep.status))}
                for op in ("logz", "mea", "sample"):
                    sel = np.array([r.op == op for r in reqs])
                    pt[f"p99_{op}_ms"] = round(float(np.percentile(lat[sel], 99)), 3)
                lens = np.array([len(r.seq) for r in reqs])
                for lo, hi in ((0, 256), (257, 512), (513, 1000)):
                    sel = (lens >= lo) & (lens <= hi)
                    if sel.any():
                        pt[f"p50_p99_len{lo}-{hi}_ms"] = [round(float(np.percentile(lat[sel], 50)), 1),
                                                          round(float(np.percentile(lat[sel], 99)), 1)]
                done = max(1, st1["done"] - st0["done"])
                pt["mean_wait_ms"] = round(1e3 * (st1["wait_s"] - st0["wait_s"]) / done, 1)
                pt["mean_batch_run_ms"] = round(1e3 * (st1["serve_s"] - st0["serve_s"]) / done, 1)
                points.append(pt)
                if frac == check_frac:
                    check = (reqs, rep.results)
        clocks = clk.summary()
    # same-as-alone check on a seeded sample of the 80 % run
    eng = Engine(P)
    reqs, results = check
    idx = np.random.default_rng(0).choice(len(reqs), min(200, len(reqs)), replace=False)
    bad = 0
    for k in idx:
        r = reqs[k]
        B = Batch([r.seq], None if r.mask is None else [r.mask])
        if r.op == "logz":
            ok = abs(float(eng.logz(B)[0]) - results[k]) <= 1e-5 * max(1.0, abs(results[k]))
        elif r.op == "mea":
            ok = eng.mea(B, r.gamma)[0] == results[k]
        else:
            ok = eng.sample(B, r.n_samples, seed=r.seed)[0] == results[k]
        bad += 0 if ok else 1
    eng.close()
    p80 = next(p for p in points if p["offered_frac"] == check_frac)
    out.update({"value": p80["p99_ms"], "saturated_folds_per_s": round(sat, 1), "points": points,
                "alone_check": {"sampled": int(len(idx)), "mismatches": bad}, "clocks": clocks})
    print(json.dumps(out), flush=True)
    return 0


def side_arm(args):
    """The other measured workloads, one JSON line each:
      logz     : 1,000 x 128 nt (default_rng(0) bases, no mask), logZ folds/s through a
                 device-resident plan (CUDA events, L2 flushed) and through logZ_batch;
                 max |logZ - FP64 logZ|; the FP64 CPU engine (oracle) on all cores.
      sampling : 4,096 sequences, lengths U{40..400} (default_rng(2)), 100 samples each,
                 samples/s with the fold included, through sample_batch (host buffers)
                 for the automatic, warp and grouped schedules.
      grad     : 512 x 300 nt, soft unpaired bonuses N(0, 0.5) (default_rng(3)),
                 gradients/s of logZ w.r.t. the 708 features and the bonuses (cf_grad +
                 the host-side tying Jacobian)."""
    import torch
    import contrafold_gpu_gb300 as cg
    from contrafold_gpu_gb300 import build as cbuild
    from contrafold_gpu_gb300.engine import CF_JOB_LOGZ, CF_JOB_LOGZ64, Batch, Engine, Plan
    cbuild.build()
    P = cg.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    alpha = np.frombuffer(b"ACGU", np.uint8)
    line = {"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic", "impl": "ours"}
    if args.workload == "logz":
        from contrafold_gpu_gb300 import workloads
        n, L = 1000, 128
        sb = workloads.logz_128(n, L)
        seqs = [bytes(r).decode() for r in sb]
        offsets = np.arange(n + 1, dtype=np.int64) * L
        d_seqs = torch.from_numpy(sb.reshape(-1).copy()).to(dev)
        eng = Engine(P)
        plan = Plan(eng, CF_JOB_LOGZ, offsets)
        d_out = torch.empty(n, dtype=torch.float32, device=dev)
        for _ in range(args.warmup):
            plan.run(d_seqs.data_ptr(), 0, d_out.data_ptr(), 6.0, stream.cuda_stream)
        plan.status()
        ms = []
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.fill_(1)
                torch.cuda.synchronize(dev)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                plan.run(d_seqs.data_ptr(), 0, d_out.data_ptr(), 6.0, stream.cuda_stream)
                e1.record(stream)
                torch.cuda.synchronize(dev)
                ms.append(e0.elapsed_time(e1))
        plan.status()
        z32 = d_out.cpu().numpy().astype(np.float64)
        p64 = Plan(eng, CF_JOB_LOGZ64, offsets)
        d64 = torch.empty(n, dtype=torch.float64, device=dev)
        p64.run(d_seqs.data_ptr(), 0, d64.data_ptr(), 6.0, stream.cuda_stream)
        p64.status()
        torch.cuda.synchronize(dev)
        err = float(np.max(np.abs(z32 - d64.cpu().numpy())))
        cg.logZ_batch(seqs[:64], P)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            cg.logZ_batch(seqs, P)
        e2e = n * args.steps / (time.perf_counter() - t0)
        from oracle import oracle as O
        O.build()
        cores = os.cpu_count() or 1
        done, tt = 0, 0.0
        while done < n and tt < 10.0:
            sl = slice(done, min(n, done + 8 * cores))
            t0 = time.perf_counter()
            O.batch(O.JOB_LOGZ64, seqs[sl], P, None, 0.0, threads=cores)
            tt += time.perf_counter() - t0
            done = sl.stop
        line.update({"metric": "logZ folds/s (1000 x 128 nt)", "value": n * len(ms) / (sum(ms) / 1e3),
                     "unit": "folds/s", "ms_per_step": statistics.mean(ms), "higher_is_better": True,
                     "dtype": "f32", "config": {"workload": "logZ, 1000 x 128 nt i.i.d. ACGU (default_rng(0)), no mask",
                                                "l2": "flushed between steps"},
                     "logz_max_abs_err_vs_fp64": err,
                     "e2e": {"value": e2e, "unit": "folds/s", "api": "contrafold_gpu_gb300.logZ_batch",
                             "h2d_bytes_per_step": n * L + 8 * (n + 1), "d2h_bytes_per_step": 4 * n},
                     "cpu_baseline": {"value": done / tt, "unit": "folds/s", "cores": cores, "kind": "port",
                                      "sample": f"first {done} sequences, FP64 inside (cpu.py:165-275 restated), "
                                                f"{cores} threads, {tt:.1f} s"},
                     "clocks": clk.summary()})
        plan.close(); p64.close(); eng.close()
    elif args.workload == "sampling":
        from contrafold_gpu_gb300 import workloads
        n, S = 4096, 100
        seqs = workloads.sampling(n)
        B = Batch(seqs)
        res = {}
        with ClockSampler(0) as clk:
            for sched in ("auto", "warp", "group"):
                eng = Engine(P)
                eng.set_schedule(sched)
                for w in range(args.warmup):
                    eng.sample(B, S, seed=w)
                ts = []
                for k in range(args.steps):
                    t0 = time.perf_counter()
                    eng.sample(B, S, seed=1000 + k)
                    ts.append(time.perf_counter() - t0)
                res[sched] = n * S / statistics.mean(ts)
                eng.close()
        line.update({"metric": "Boltzmann samples/s (fold included), 4096 seqs x U{40..400} nt x 100 samples",
                     "value": res["auto"], "unit": "samples/s", "higher_is_better": True, "dtype": "f32",
                     "schedules": res, "config": {"workload": "sampling, 4096 x U{40..400} nt (default_rng(2)), "
                                                              "100 samples each, Philox (seed, seq, sample)",
                                                  "api": "Engine.sample (host buffers, copies timed)"},
                     "e2e": {"value": res["auto"], "unit": "samples/s", "h2d_bytes_per_step": int(B.total + 8 * (n + 1)),
                             "d2h_bytes_per_step": int(B.total * S)},
                     "clocks": clk.summary()})
    else:
        from contrafold_gpu_gb300 import grad
        from contrafold_gpu_gb300 import workloads
        n, L = 512, 300
        seqs, bonus = workloads.grad_300(n, L)
        eng = Engine(P)
        for _ in range(args.warmup):
            grad.logz_grad(seqs, None, list(bonus), engine=eng)
        ts = []
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                t0 = time.perf_counter()
                res = grad.logz_grad(seqs, None, list(bonus), engine=eng)
                ts.append(time.perf_counter() - t0)
        # sum_k P(k unpaired) + 2 E[#pairs] = L; its float32 residual, relative to L
        ident = float(np.max([abs(res.d_bonus[b].sum() - (L - 2 * res.d_blob[b, 0:25].sum())) for b in range(n)])) / L
        from contrafold_gpu_gb300.engine import grad_arena_bytes
        line.update({"metric": "logZ gradients/s (708 features + per-position bonus), 512 x 300 nt",
                     "value": n / statistics.mean(ts), "unit": "gradients/s", "higher_is_better": True,
                     "dtype": "f32 tables, fixed-point (2^-62) counts", "ms_per_step": 1e3 * statistics.mean(ts),
                     "memory_per_sequence_bytes": {"300nt_auto": grad_arena_bytes(300, 0),
                                                   "1000nt_every8": grad_arena_bytes(1000, 8),
                                                   "1000nt_all": grad_arena_bytes(1000, 1),
                                                   "3000nt_every8": grad_arena_bytes(3000, 8)},
                     "config": {"workload": "gradient, 512 x 300 nt i.i.d. ACGU, bonuses N(0,0.5) (default_rng(3))",
                                "api": "grad.logz_grad (host buffers; tying Jacobian on the host)"},
                     "identity_max_rel_err": ident, "clocks": clk.summary()})
        eng.close()
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=10000)
    ap.add_argument("--L", type=int, default=200)
    ap.add_argument("--workload", choices=["mea", "bpp", "mfe", "serving", "logz", "sampling", "grad"], default="mea",
                    help="mea: the headline 200-nt MEA batch; bpp / mfe: the other decoders of the same "
                         "batch; serving: the open-loop request-stream sweep; logz / sampling / grad: the other "
                         "measured workloads")
    ap.add_argument("--workers", type=int, default=6, help="serving: engines / worker threads")
    ap.add_argument("--long-workers", type=int, default=2, help="serving: workers that take long requests")
    ap.add_argument("--long-len", type=int, default=256, help="serving: buckets above this length are long")
    ap.add_argument("--edges", type=int, nargs="+", default=[96, 192, 256, 384, 640],
                    help="serving: length-bucket upper edges")
    ap.add_argument("--max-batch-cost", type=float, default=0.0,
                    help="serving: cap on a batch's predicted work, sum of L^3 (0 = none)")
    ap.add_argument("--max-batch-arena", type=int, default=0,
                    help="serving: cap on a batch's device arena bytes (0 = none)")
    ap.add_argument("--serve-n", type=int, default=20000, help="serving: requests of the saturation run")
    ap.add_argument("--serve-seconds", type=float, default=4.0, help="serving: seconds of arrivals per load point")
    ap.add_argument("--serve-fracs", type=float, nargs="+", default=[0.2, 0.5, 0.8, 0.9])
    args = ap.parse_args()
    if args.workload == "serving":
        return serving_arm(args)
    if args.workload in ("logz", "sampling", "grad"):
        return side_arm(args)
    if args.workload in ("bpp", "mfe"):
        return decoder_arm(args)
    if args.impl == "reference":
        return reference_arm(args)
    return our_arm(args)


if __name__ == "__main__":
    sys.exit(main())
