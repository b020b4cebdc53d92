"""Batch RNA folding CLI (drop-in for the reference's `gpu-contrafold`, gpu_contrafold/cli.py).

    gpu-contrafold GGGGAAAACCCC                  # one sequence -> MEA structure (dot-bracket)
    gpu-contrafold GGGGAAAACCCC --gamma 4        # MEA with a custom tradeoff
    gpu-contrafold GGGGAAAACCCC --viterbi        # max-probability (Viterbi/MAP) structure
    gpu-contrafold GGGGAAAACCCC --sample 10      # 10 Boltzmann samples
    gpu-contrafold GGGGAAAACCCC --logz           # partition function (logZ)
    gpu-contrafold seqs.jsonl -o out.jsonl       # batch (JSONL in/out)
    gpu-contrafold seqs.fa --parens out.parens   # structures also as a CONTRAfold parens file
    gpu-contrafold seqs.fa --posteriors 1e-5 out.post   # sparse posterior file (CONTRAfold format)

Same arguments, input sniffing, mask validation, mode precedence and output
format as the reference (cli.py:88-230).  The difference is where the work
runs: MEA and Viterbi structures are folded in length-sorted batches on the
GPU (the reference folds them one record at a time on the CPU,
cli.py:188-193), and every mode goes through the same engine.

JSONL input (one object per line):
    {"id": "rna1", "seq": "GGGGAAAACCCC", "constrain": [0,0,0,1,0,0,0,0,0,0,0,0]}
  - seq        (required) RNA sequence; non-ACGU is treated as N (cannot pair).
  - id         (optional) echoed to output; defaults to the 0-based index.
  - constrain  (optional) per-base 0/1 hard-constraint mask, length == len(seq),
               1 = forced unpaired. Accepts a list [0,0,1,...] or a string "001...".

Output: a single literal sequence prints structures to stdout (one per line);
file input (or any -o) writes JSONL ({"id","structure"}, or {"id","samples":[...]}
for --sample N, or {"id","logZ"} for --logz), input order preserved.

--parens FILE and --posteriors CUTOFF FILE take the CONTRAfold binary's
`predict` options of the same names (the reference reads those files in
gpu_contrafold/reference.py:61-132): the structures, and the base-pair
posteriors >= CUTOFF, written in that binary's file formats (`formats.py`).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

_SEQ_CHARS = set("ACGUTN")


def _parse_jsonl(path):
    recs = []
    with open(path) as fh:
        for ln, line in enumerate(fh):
            line = line.strip()
            if not line:
                continue
            try:
                obj = json.loads(line)
            except json.JSONDecodeError as e:
                raise SystemExit(f"line {ln}: invalid JSON ({e})")
            if "seq" not in obj or not obj["seq"]:
                raise SystemExit(f"line {ln}: missing required field 'seq'")
            recs.append((obj.get("id", ln), str(obj["seq"]).strip().upper(), obj.get("constrain")))
    return recs


def _parse_fasta(path):
    recs, rid, cur = [], None, []
    with open(path) as fh:
        for line in fh:
            line = line.rstrip("\n")
            if line.startswith(">"):
                if cur:
                    recs.append((rid, "".join(cur).upper(), None))
                    cur = []
                rid = line[1:].strip() or len(recs)
            elif line.strip():
                cur.append(line.strip())
    if cur:
        recs.append((rid, "".join(cur).upper(), None))
    return recs


def _parse_seq_lines(path):
    recs = []
    with open(path) as fh:
        for i, line in enumerate(fh):
            s = line.strip().upper()
            if s:
                recs.append((i, s, None))
    return recs


def load_records(src):
    """(records, from_file); records are (id, seq, constrain) (cli.py:88-105)."""
    if os.path.isfile(src):
        head = ""
        with open(src) as fh:
            for line in fh:
                if line.strip():
                    head = line.strip()[0]
                    break
        if head == "{":
            return _parse_jsonl(src), True
        if head == ">":
            return _parse_fasta(src), True
        return _parse_seq_lines(src), True
    seq = src.strip().upper()
    if seq and all(c in _SEQ_CHARS for c in seq):
        return [(0, seq, None)], False
    raise SystemExit(f"'{src}' is not an existing file nor a valid RNA sequence (ACGUTN)")


def build_mask(seq, constrain, where=""):
    """Per-base 0/1 mask (1 = forced unpaired) -> int8 array, or None (cli.py:108-124)."""
    if not constrain:
        return None
    L = len(seq)
    bits = [1 if c == "1" else 0 for c in constrain] if isinstance(constrain, str) else list(constrain)
    if len(bits) != L:
        raise SystemExit(f"{where}constrain length {len(bits)} != seq length {L}")
    m = np.zeros(L, np.int8)
    for i, b in enumerate(bits):
        if b not in (0, 1):
            raise SystemExit(f"{where}constrain[{i}] = {b!r}, expected 0 or 1")
        m[i] = b
    return m


def fold(records, P, mode="mea", sample_n=0, with_logz=False, gamma=6.0, chunk=4096, seed=0):
    """Fold records on the GPU in length-sorted chunks; results in input order.

    Sampling chunk c0 uses seed + c0 as the reference does (cli.py:139-140)."""
    from . import gpu
    n = len(records)
    seqs = [r[1] for r in records]
    masks = [build_mask(r[1], r[2], where=f"id={r[0]!r}: ") for r in records]
    order = sorted(range(n), key=lambda k: len(seqs[k]))
    logz, samples, structures = [None] * n, [None] * n, [None] * n
    for c0 in range(0, n, chunk):
        idx = order[c0:c0 + chunk]
        sub = [seqs[k] for k in idx]
        fl = [masks[k] for k in idx]
        if mode == "sample":
            for k, r in zip(idx, gpu.sample_batch(sub, P, sample_n, forced_list=fl, seed=seed + c0)):
                samples[k] = r
            if with_logz:
                for k, z in zip(idx, gpu.logZ_batch(sub, P, forced_list=fl)):
                    logz[k] = z
        elif mode == "logz":
            for k, z in zip(idx, gpu.logZ_batch(sub, P, forced_list=fl)):
                logz[k] = z
        elif mode == "mfe":
            for k, st in zip(idx, gpu.mfe_batch(sub, P, forced_list=fl)):
                structures[k] = st
        else:
            for k, st in zip(idx, gpu.mea_batch(sub, P, gamma=gamma, forced_list=fl)):
                structures[k] = st
    return logz, samples, structures


def posteriors(records, P, chunk=4096):
    """Base-pair probability matrices of the records (GPU, length-sorted
    chunks), in input order."""
    from . import gpu
    seqs = [r[1] for r in records]
    masks = [build_mask(r[1], r[2], where=f"id={r[0]!r}: ") for r in records]
    order = sorted(range(len(records)), key=lambda k: len(seqs[k]))
    out = [None] * len(records)
    for c0 in range(0, len(records), chunk):
        idx = order[c0:c0 + chunk]
        for k, m in zip(idx, gpu.bpp_batch([seqs[k] for k in idx], P, forced_list=[masks[k] for k in idx])):
            out[k] = m
    return out


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    if argv and argv[0] == "fold":          # back-compat: optional 'fold' subcommand
        argv = argv[1:]
    parser = argparse.ArgumentParser(prog="gpu-contrafold", description=__doc__,
                                     formatter_class=argparse.RawDescriptionHelpFormatter)
    parser.add_argument("input", help="RNA sequence, or path to a JSONL/FASTA/sequence-per-line file")
    parser.add_argument("-o", "--output", default=None, help="output JSONL (default: stdout)")
    parser.add_argument("--sample", type=int, default=0, metavar="N",
                        help="draw N Boltzmann samples per sequence (default: MEA structure)")
    parser.add_argument("--viterbi", "--mfe", action="store_true", dest="viterbi",
                        help="max-probability (Viterbi/MAP) structure instead of MEA")
    parser.add_argument("--gamma", type=float, default=6.0, metavar="G",
                        help="MEA sensitivity/specificity tradeoff (default: 6); ignored with --viterbi")
    parser.add_argument("--logz", action="store_true",
                        help="emit the partition function (logZ) instead of a structure")
    parser.add_argument("--chunk", type=int, default=4096, help="sequences per GPU launch")
    parser.add_argument("--threads", type=int, default=128,
                        help="accepted for compatibility; the engine picks its own launch shape")
    parser.add_argument("--seed", type=int, default=0, help="RNG seed for sampling")
    parser.add_argument("--parens", default=None, metavar="FILE",
                        help="also write the structures as a CONTRAfold parens file (>id, sequence, structure)")
    parser.add_argument("--posteriors", nargs=2, default=None, metavar=("CUTOFF", "FILE"),
                        help="also write base-pair posteriors >= CUTOFF in CONTRAfold's sparse format")
    args = parser.parse_args(argv)
    cutoff = None
    if args.posteriors is not None:
        try:
            cutoff = float(args.posteriors[0])
        except ValueError:
            raise SystemExit(f"--posteriors: cutoff {args.posteriors[0]!r} is not a number")

    records, from_file = load_records(args.input)
    if not records:
        raise SystemExit("no sequences in input")
    # mode precedence: sample > logz > viterbi > mea (cli.py:177-184)
    if args.sample:
        mode = "sample"
    elif args.logz:
        mode = "logz"
    elif args.viterbi:
        mode = "mfe"
    else:
        mode = "mea"
    if args.parens and mode not in ("mea", "mfe"):
        raise SystemExit("--parens writes structures: not with --sample or --logz")

    from .params import load
    P = load()
    logz, samples, structures = fold(records, P, mode=mode, sample_n=args.sample, with_logz=args.logz,
                                     gamma=args.gamma, chunk=args.chunk, seed=args.seed)
    from . import formats
    if args.parens:
        formats.write_parens_file(args.parens, [(r[0], r[1], st) for r, st in zip(records, structures)])
    if args.posteriors is not None:
        mats = posteriors(records, P, chunk=args.chunk)
        formats.write_posteriors_file(args.posteriors[1], [(r[0], r[1], m) for r, m in zip(records, mats)], cutoff)

    if not from_file and not args.output:
        if mode in ("mfe", "mea"):
            print(structures[0])
        elif mode == "sample":
            if args.logz:
                print(f"# logZ = {logz[0]:.6f}")
            for db in samples[0]:
                print(db)
        else:
            print(f"{logz[0]:.6f}")
        return

    out = open(args.output, "w") if args.output else sys.stdout
    try:
        for k, (rid, _seq, _con) in enumerate(records):
            rec = {"id": rid}
            if mode in ("mfe", "mea"):
                rec["structure"] = structures[k]
            elif mode == "sample":
                if args.logz:
                    rec["logZ"] = logz[k]
                rec["samples"] = samples[k]
            else:
                rec["logZ"] = logz[k]
            out.write(json.dumps(rec) + "\n")
    finally:
        if args.output:
            out.close()
    if args.output:
        print(f"[gpu-contrafold] wrote {len(records)} records -> {args.output}", file=sys.stderr)


if __name__ == "__main__":
    main()
