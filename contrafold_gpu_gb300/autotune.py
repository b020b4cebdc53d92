"""Schedule autotuner for the batched path.

For each length bucket it times a synthetic MEA batch (i.i.d. ACGU, 10 %
forced-unpaired mask) on the GPU under every schedule the engine offers --
the persistent warp-per-sequence kernel and the persistent CTA-per-sequence
fused kernel at 1..4 resident CTAs per SM -- and reports folds/s per choice
and the best one per bucket.  Every schedule computes identical results; only
speed differs.  The engine's built-in schedule table (cf_engine.cu,
default_tuning) was set from these measurements.

    python -m contrafold_gpu_gb300.autotune [--lengths 50,100,200,300,400] [--json out.json]
    python -m contrafold_gpu_gb300.autotune --lengths 100,200 --batch-sizes 256,1024,4096
    python -m contrafold_gpu_gb300.autotune --latency --lengths 150,400,600,1000 --batch-sizes 1,16,32

--latency times small batches of long sequences (ms per batch) on the grouped
and the cluster schedules and, with --phase-timing, the grouped schedule's
per-phase kernels; --mask-frac sets the forced-unpaired fraction (1.0: no
pairable cell, the bifurcation chains alone).

--write-table FILE runs the sweeps that decide the automatic schedule and
writes the engine's schedule table (include/contrafold_gb300.h,
cf_engine_load_tuning): for mixed-length batches (lengths uniform in
[Lmax/2, Lmax]) of each --lengths x --batch-sizes cell, the faster of the
warp and grouped schedules (MEA folds/s); for small batches of long
sequences, the grouped or the cluster schedule (ms per batch).  The engine
reads the table through Engine.load_tuning(FILE) or, at creation, from the
environment variable CONTRAFOLD_GB300_TUNING.

    python -m contrafold_gpu_gb300.autotune --write-table tuning.txt \
        --lengths 80,160,256 --batch-sizes 512,2048,8192 --long-lengths 512,768 --long-batches 8,38
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def _batch_bytes(n, L, seed, mask_frac=0.1):
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, 4, size=(n, L), dtype=np.int8)
    seq = np.frombuffer(b"ACGU", np.uint8)[idx].reshape(-1).copy()
    mask = (rng.random((n, L)) < mask_frac).astype(np.uint8).reshape(-1)
    return seq, mask


def time_latency(P, L, n, kind, job="mea", mask_frac=0.1, phases=False, reps=3):
    """Best wall time (ms) of one batch of n sequences of L nt on schedule
    `kind`, and the per-phase device times when `phases` (per-phase kernels)."""
    import torch
    from .engine import CF_JOB_LOGZ, CF_JOB_MEA, Engine, Plan
    seq, mask = _batch_bytes(n, L, 7, mask_frac)
    dev = torch.device("cuda", 0)
    d_seq = torch.from_numpy(seq).to(dev)
    d_mask = torch.from_numpy(mask).to(dev)
    d_out = torch.empty(n * L if job == "mea" else 4 * n, dtype=torch.uint8, device=dev)
    eng = Engine(P)
    eng.set_schedule(kind)
    plan = Plan(eng, CF_JOB_MEA if job == "mea" else CF_JOB_LOGZ, np.arange(n + 1, dtype=np.int64) * L)
    plan.set_timing(phases)
    stream = torch.cuda.Stream(dev)
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        plan.run(d_seq.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), 6.0, stream.cuda_stream)
        plan.status()
        best = min(best, (time.perf_counter() - t0) * 1e3)
    ph = [round(float(x), 2) for x in plan.phase_ms()] if phases else None
    plan.close()
    eng.close()
    return best, ph


def time_schedule(P, L, n, kind, ctas, reps=3, job="mea", group=0):
    import torch
    from .engine import CF_JOB_LOGZ, CF_JOB_MEA, Engine, Plan
    seq, mask = _batch_bytes(n, L, 7)
    dev = torch.device("cuda", 0)
    d_seq = torch.from_numpy(seq).to(dev)
    d_mask = torch.from_numpy(mask).to(dev)
    d_out = torch.empty(n * L if job == "mea" else 4 * n, dtype=torch.uint8, device=dev)
    eng = Engine(P, mode="plain" if kind == "plain" else "batched")
    if kind != "plain":
        eng.set_schedule(kind, ctas)
    if group:
        eng.set_group(group)
    plan = Plan(eng, CF_JOB_MEA if job == "mea" else CF_JOB_LOGZ, np.arange(n + 1, dtype=np.int64) * L)
    stream = torch.cuda.Stream(dev)
    plan.run(d_seq.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), 6.0, stream.cuda_stream)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.run(d_seq.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), 6.0, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    plan.status()
    plan.close()
    eng.close()
    return n / (best / 1000.0)


def _mixed_batch(n, Lmax, seed):
    rng = np.random.default_rng(seed)
    lens = rng.integers(max(1, Lmax // 2), Lmax + 1, n)
    lens[0] = Lmax
    seqs = [np.frombuffer(b"ACGU", np.uint8)[rng.integers(0, 4, int(L))].tobytes().decode() for L in lens]
    masks = [(rng.random(int(L)) < 0.1).astype(np.int8) for L in lens]
    return seqs, masks


def time_mixed(P, n, Lmax, kind, reps=2):
    """MEA folds/s of a mixed-length batch on schedule `kind` (host buffers, best of reps)."""
    from .engine import Batch, Engine
    seqs, masks = _mixed_batch(n, Lmax, 11)
    B = Batch(seqs, masks)
    eng = Engine(P)
    eng.set_schedule(kind)
    eng.mea(B, 6.0)
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        eng.mea(B, 6.0)
        best = min(best, time.perf_counter() - t0)
    eng.close()
    return n / best


def time_sampling(P, n, Lmax, group, n_samples=100, reps=2):
    """Samples/s of a mixed-length batch on the grouped schedule with `group`
    sequences per CTA (0 = the engine's choice), fold included, host buffers."""
    from .engine import Batch, Engine
    seqs, _ = _mixed_batch(n, Lmax, 12)
    B = Batch(seqs)
    eng = Engine(P)
    eng.set_schedule("group")
    eng.set_group(group)
    eng.sample(B, n_samples, seed=1)
    best = float("inf")
    for k in range(reps):
        t0 = time.perf_counter()
        eng.sample(B, n_samples, seed=2 + k)
        best = min(best, time.perf_counter() - t0)
    eng.close()
    return n * n_samples / best


def tuning_rows(P, lengths, batch_sizes, long_lengths, long_batches, log=print):
    """Measure and return the schedule table as text rows (first match wins)."""
    rows = ["# contrafold-gb300 schedule table, written by contrafold_gpu_gb300.autotune --write-table",
            "# min_len max_len min_batch max_batch uniform jobs schedule group ctas_per_sm"]
    # long sequences, small batches: cluster vs grouped latency (longer minimum
    # lengths first: the first matching row wins)
    for Lo in sorted(long_lengths, reverse=True):
        for n in sorted(long_batches):
            g_ms, _ = time_latency(P, Lo, n, "group")
            c_ms, _ = time_latency(P, Lo, n, "cluster")
            best = "cluster" if c_ms < g_ms else "group"
            log(f"long L>={Lo} n<={n}: group {g_ms:.1f} ms cluster {c_ms:.1f} ms -> {best}")
            rows.append(f"{Lo} 32767 1 {n} any logz,bpp,mea,sample {best} 0 0")
    # mixed lengths: warp vs grouped throughput, most specific rows first
    prev = 0
    for Lmax in sorted(lengths):
        cells = []
        for n in sorted(batch_sizes):
            w = time_mixed(P, n, Lmax, "warp")
            g = time_mixed(P, n, Lmax, "group")
            best = "warp" if w > g else "group"
            log(f"mixed {prev + 1}-{Lmax} nt n={n}: warp {w:.0f} group {g:.0f} folds/s -> {best}")
            cells.append((n, best))
        for n, best in sorted(cells, reverse=True):
            rows.append(f"0 {Lmax} {n} 0 mixed logz,bpp,mea {best} 0 0")
        prev = Lmax
    # sampling of mixed lengths (the fold is an inside only): sequences per CTA
    n = max(batch_sizes)
    for Lmax in sorted(lengths):
        rates = {g: time_sampling(P, n, Lmax, g) for g in (0, 2, 3, 4, 6)}
        g = max(rates, key=rates.get)
        log(f"sampling mixed <= {Lmax} nt n={n}: " + " ".join(f"g{k} {v / 1e6:.3f}M" for k, v in rates.items())
            + f" -> {g}")
        if g:
            rows.append(f"0 {Lmax} {n} 0 mixed sample group {g} 0")
    return rows


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--lengths", default="50,100,200,300,400")
    ap.add_argument("--folds", type=float, default=2.5e10, help="work per bucket ~ folds * L^3 (sizes n)")
    ap.add_argument("--job", default="mea", choices=["mea", "logz"])
    ap.add_argument("--json", default=None)
    ap.add_argument("--batch-sizes", default=None,
                    help="comma list: time the warp and grouped schedules at each (length, batch size) -- the "
                         "batch size from which the engine takes the warp kernel (auto_warp_min_batch)")
    ap.add_argument("--groups", default=None,
                    help="comma list: time the grouped schedule with each number of sequences per CTA at every "
                         "length (batch sized as for the schedule table) -- the engine's group_for_length table")
    ap.add_argument("--latency", action="store_true",
                    help="ms per small batch on the grouped and cluster schedules (lengths x --batch-sizes)")
    ap.add_argument("--mask-frac", type=float, default=0.1, help="--latency: forced-unpaired fraction")
    ap.add_argument("--phase-timing", action="store_true", help="--latency: grouped per-phase kernel times")
    ap.add_argument("--write-table", default=None, metavar="FILE",
                    help="measure and write the engine's schedule table (--lengths, --batch-sizes, --long-lengths, "
                         "--long-batches)")
    ap.add_argument("--long-lengths", default="512,768")
    ap.add_argument("--long-batches", default="8,38")
    args = ap.parse_args()
    from . import load
    P = load()
    if args.write_table:
        ints = lambda x: [int(v) for v in x.split(",")]
        rows = tuning_rows(P, ints(args.lengths), ints(args.batch_sizes or "512,2048,8192"),
                           ints(args.long_lengths), ints(args.long_batches))
        with open(args.write_table, "w") as fh:
            fh.write("\n".join(rows) + "\n")
        print(f"wrote {len(rows) - 2} rows -> {args.write_table}")
        return rows
    if args.latency:
        table = {}
        for L in [int(x) for x in args.lengths.split(",")]:
            for n in [int(x) for x in (args.batch_sizes or "1").split(",")]:
                g_ms, ph = time_latency(P, L, n, "group", args.job, args.mask_frac, args.phase_timing)
                c_ms, _ = time_latency(P, L, n, "cluster", args.job, args.mask_frac)
                table[f"{L}x{n}"] = {"group_ms": g_ms, "cluster_ms": c_ms, "group_phase_ms": ph}
                print(f"L={L:4d} n={n:4d} group {g_ms:8.2f} ms  cluster {c_ms:8.2f} ms"
                      + (f"  group phases {ph}" if ph else ""), flush=True)
        if args.json:
            with open(args.json, "w") as fh:
                json.dump(table, fh, indent=1)
        return table
    if args.groups:
        table = {}
        for L in [int(x) for x in args.lengths.split(",")]:
            n = int(max(304, min(20000, args.folds / L ** 3)))
            row = {g: time_schedule(P, L, n, "group", 0, job=args.job, group=int(g)) for g in args.groups.split(",")}
            best = max(row, key=row.get)
            table[L] = {"n": n, "folds_per_s": row, "best": int(best)}
            print(f"L={L:4d} n={n:6d} " + " ".join(f"g{g}:{v:9.1f}" for g, v in row.items()) + f" -> group {best}",
                  flush=True)
        if args.json:
            with open(args.json, "w") as fh:
                json.dump(table, fh, indent=1)
        return table
    if args.batch_sizes:
        table = {}
        for L in [int(x) for x in args.lengths.split(",")]:
            for n in [int(x) for x in args.batch_sizes.split(",")]:
                row = {k: time_schedule(P, L, n, k, 0, job=args.job) for k in ("warp", "group")}
                table[f"{L}x{n}"] = row
                print(f"L={L:4d} n={n:6d} warp {row['warp']:10.1f} group {row['group']:10.1f} folds/s "
                      f"-> {'warp' if row['warp'] > row['group'] else 'group'}", flush=True)
        if args.json:
            with open(args.json, "w") as fh:
                json.dump(table, fh, indent=1)
        return table
    schedules = [("plain", 0), ("warp", 0), ("group", 0), ("cta", 3), ("cta", 4)]
    table = {}
    for L in [int(x) for x in args.lengths.split(",")]:
        n = int(max(304, min(20000, args.folds / L ** 3)))
        row = {}
        for kind, ctas in schedules:
            t0 = time.time()
            key = f"{kind}{ctas}" if ctas else kind
            row[key] = time_schedule(P, L, n, kind, ctas, job=args.job)
            print(f"L={L:4d} n={n:6d} {key:6s}: {row[key]:10.1f} folds/s ({time.time() - t0:.1f}s)", flush=True)
        best = max((v, k) for k, v in row.items() if k != "plain")
        table[L] = {"n": n, "folds_per_s": row, "best": best[1], "speedup_vs_plain": best[0] / row["plain"]}
        print(f"L={L}: best {best[1]} {best[0]:.0f} folds/s = {best[0] / row['plain']:.2f}x plain", flush=True)
    if args.json:
        with open(args.json, "w") as fh:
            json.dump(table, fh, indent=1)
    return table


if __name__ == "__main__":
    main()
