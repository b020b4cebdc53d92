"""Batch RNA folding CLI (drop-in for the reference's `gpu-contrafold`, gpu_contrafold/cli.py).

    gpu-contrafold GGGGAAAACCCC                  # one sequence -> MEA structure (dot-bracket)
    gpu-contrafold GGGGAAAACCCC --gamma 4        # MEA with a custom tradeoff
    gpu-contrafold GGGGAAAACCCC --viterbi        # max-probability (Viterbi/MAP) structure
    gpu-contrafold GGGGAAAACCCC --sample 10      # 10 Boltzmann samples
    gpu-contrafold GGGGAAAACCCC --logz           # partition function (logZ)
    gpu-contrafold seqs.jsonl -o out.jsonl       # batch (JSONL in/out)
    gpu-contrafold seqs.fa --parens out.parens   # structures also as a CONTRAfold parens file
    gpu-contrafold seqs.fa --posteriors 1e-5 out.post   # sparse posterior file (CONTRAfold format)

Same arguments, input behaviour (below), mode precedence and output format
as the reference (cli.py:88-230).  The difference is where the work
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
from typing import Any, Iterable, List, NamedTuple, Tuple

import numpy as np

# Input behaviour (kept for drop-in use; the reference's CLI accepts the same):
#  * the argument names an existing file, or else is itself one sequence of the
#    letters A C G U T N in any case (anything else is an error exit);
#  * a file's format is decided by the first character of its first non-blank
#    line: "{" JSON lines, ">" FASTA, anything else one sequence per line;
#  * JSON lines: one object per non-blank line with "seq" (required, non-empty)
#    and optional "id" (default: the 0-based line number) and "constrain";
#    malformed JSON or a missing "seq" is an error exit naming the line;
#  * FASTA: a ">" line opens a record named by the rest of the line (or, when
#    that is empty, by how many records precede it); its sequence is the
#    following non-blank lines joined; a record without sequence is dropped;
#  * sequence per line: every non-blank line is a record named by its 0-based
#    line number;
#  * sequences are upper-cased and stripped of surrounding white space;
#  * "constrain" is a 0/1 list or a string in which "1" marks a forced-unpaired
#    position (any other character is 0); it must have one entry per base and
#    list entries must be 0 or 1 -- otherwise an error exit.
_NUCLEOTIDES = frozenset("ACGUTN")


class Record(NamedTuple):
    id: Any
    seq: str
    constrain: Any = None


def _read_jsonl(numbered: Iterable[Tuple[int, str]]) -> List[Record]:
    out: List[Record] = []
    for lineno, text in numbered:
        if not text.strip():
            continue
        try:
            obj = json.loads(text)
        except json.JSONDecodeError as err:
            raise SystemExit(f"line {lineno}: invalid JSON ({err})")
        seq = obj.get("seq") if isinstance(obj, dict) else None
        if not seq:
            raise SystemExit(f"line {lineno}: missing required field 'seq'")
        out.append(Record(obj.get("id", lineno), str(seq).strip().upper(), obj.get("constrain")))
    return out


def _read_fasta(numbered: Iterable[Tuple[int, str]]) -> List[Record]:
    out: List[Record] = []
    name: Any = None
    parts: List[str] = []

    def close():
        if parts:
            out.append(Record(name, "".join(parts).upper()))

    for _, text in numbered:
        if text.startswith(">"):
            close()
            parts = []
            name = text[1:].strip() or len(out)
        elif text.strip():
            parts.append(text.strip())
    close()
    return out


def _read_lines(numbered: Iterable[Tuple[int, str]]) -> List[Record]:
    return [Record(lineno, text.strip().upper()) for lineno, text in numbered if text.strip()]


_READERS = {"{": _read_jsonl, ">": _read_fasta}


def load_records(src: str):
    """(records, from_file): the records (id, seq, constrain) named by `src`,
    a file path or a literal sequence (input behaviour above)."""
    if os.path.isfile(src):
        with open(src) as fh:
            numbered = [(k, line.rstrip("\n")) for k, line in enumerate(fh)]
        first = next((t.strip()[0] for _, t in numbered if t.strip()), "")
        return _READERS.get(first, _read_lines)(numbered), True
    seq = src.strip().upper()
    if seq and frozenset(seq) <= _NUCLEOTIDES:
        return [Record(0, seq)], False
    raise SystemExit(f"'{src}' is not an existing file nor a valid RNA sequence (ACGUTN)")


def build_mask(seq: str, constrain, where: str = ""):
    """int8 forced-unpaired mask (1 = forced) from a record's "constrain", or
    None when it has none (input behaviour above)."""
    if constrain is None or len(constrain) == 0:
        return None
    if isinstance(constrain, str):
        bits = [int(ch == "1") for ch in constrain]
    else:
        bits = list(constrain)
    if len(bits) != len(seq):
        raise SystemExit(f"{where}constrain length {len(bits)} != seq length {len(seq)}")
    bad = next((k for k, b in enumerate(bits) if b not in (0, 1)), None)
    if bad is not None:
        raise SystemExit(f"{where}constrain[{bad}] = {bits[bad]!r}, expected 0 or 1")
    return np.asarray(bits, np.int8)


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
