"""Generate the golden fixtures from the reference engine itself.

Imports the reference's CPU engine (gpu_contrafold/cpu.py, read from the
reference checkout given by the required --ref argument) under an identity
`numba.njit` stub -- numba is not installed here, so the reference runs as
plain Python/numpy with the same float32/float64 scalar semantics -- and
records, for seeded inputs:

  * the tied float64 parameter blob (cpu.load, cpu.py:40-135);
  * FP64 logZ from cpu.inside (cpu.py:165-275), masks included;
  * Viterbi structures from cpu.mfe (cpu.py:505-519);
  * MEA structures from cpu.mea at several gammas (cpu.py:932-941);
  * the FP32 posterior matrix from cpu.posterior (cpu.py:583-820): the full
    bytes for short sequences, a SHA-256 of the float32 bytes for the rest;
  * the reference's own literal known answers (GGGGAAAACCCC, README.md:101,104)
    and the sequences of its validation script (tests/test_validation.py:15-27).

Run once in a container that has the reference checkout:
    python tests/golden/make_golden.py --ref <reference checkout> [--jobs 8]
The output, tests/golden/golden.json (+ params_blob64.npy), is committed; the
tests read only those files.

    python tests/golden/make_golden.py --ref <reference checkout> --exhaustive
writes tests/golden/exhaustive.json.gz instead: every ACGU sequence of 1-5 nt
without a mask and every (sequence, mask) pair of 1-4 nt, each with FP64 logZ,
the Viterbi and MEA (gamma 6) structures and the first 16 hex digits of the
SHA-256 of its float32 posterior matrix.

    python tests/golden/make_golden.py --ref <reference checkout> --long
writes tests/golden/long.json: seven seeded sequences of 300-600 nt (masks
Bernoulli 0.1 / 0.3 on some, N on one) with the same fields as golden.json
(minutes per case: the reference runs as plain Python).

    python tests/golden/make_golden.py --ref <reference checkout> --xlong
writes tests/golden/xlong.json: one 800-nt and one 1,000-nt sequence (the
latter with a Bernoulli 0.1 mask), about an hour of pure Python.

    python tests/golden/make_golden.py --ref <reference checkout> --mea200 500
writes tests/golden/mea200_subset.json.gz: the first 500 sequences of the
10,000 x 200 nt MEA workload (contrafold_gpu_gb300.workloads.mea_200: bases
default_rng(0), Bernoulli(0.1) mask default_rng(1)), each with FP64 logZ, the
Viterbi and MEA (gamma 6) structures and the posterior digest (about half an
hour of pure Python on 8 cores).
"""
from __future__ import annotations

import argparse
import base64
import gzip
import hashlib
import importlib.util
import itertools
import json
import multiprocessing as mp
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

_STUB = '''
def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    def deco(f):
        return f
    return deco
'''

_REF = None
_P = None


def load_reference(ref_root):
    """Import <ref_root>/gpu_contrafold/cpu.py with an identity numba.njit."""
    stub_dir = tempfile.mkdtemp(prefix="numba_stub_")
    os.makedirs(os.path.join(stub_dir, "numba"))
    with open(os.path.join(stub_dir, "numba", "__init__.py"), "w") as fh:
        fh.write(_STUB)
    sys.path.insert(0, stub_dir)
    path = os.path.join(ref_root, "gpu_contrafold", "cpu.py")
    spec = importlib.util.spec_from_file_location("ref_cpu", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _init(ref_root):
    global _REF, _P
    _REF = load_reference(ref_root)
    _P = _REF.load()


def _run_case(args):
    seq, mask, gammas, want_post_bytes = args
    R, P = _REF, _P
    L = len(seq)
    s, _ = R.encode(seq)
    fo = np.zeros(L + 2, dtype=np.int64)
    if mask is not None:
        for k in range(L):
            fo[k + 1] = int(mask[k])
    t0 = time.time()
    z64 = R.inside(s, L, fo, P["bp"], P["stack"], P["tm"], P["hc"], P["dl"], P["dr"],
                   P["hp_cum"], P["cs"], P["i11"], P["b01"], P["mb"], P["mu"], P["mp"],
                   P["eu"], P["ep"], R._CANON)
    mfe = R.mfe(seq, P, mask)
    _s, _L, _fo, POST = R._posterior(seq, P, mask)
    f = R._params_f32(P)
    meas = {}
    for g in gammas:
        pair = R.mea_decode(POST, L, _fo, R._CANON, _s, np.float32(g))
        ch = ["."] * L
        for t in range(1, L + 1):
            if pair[t] > t:
                ch[t - 1] = "("
                ch[pair[t] - 1] = ")"
        meas[repr(float(g))] = "".join(ch)
    post = np.ascontiguousarray(POST, dtype=np.float32)
    rec = {
        "seq": seq,
        "mask": None if mask is None else "".join("1" if int(x) else "0" for x in mask),
        "logz64": float(z64),
        "mfe": mfe,
        "mea": meas,
        "post_sha256": hashlib.sha256(post.tobytes()).hexdigest(),
        "post_sum": float(post.astype(np.float64).sum()),
        "seconds": round(time.time() - t0, 2),
    }
    if want_post_bytes:
        rec["post_b64"] = base64.b64encode(post.tobytes()).decode("ascii")
    del f
    return rec


def _run_small(args):
    """Compact record of one exhaustive case: seq, mask bits, logZ, Viterbi,
    MEA (gamma 6), posterior digest."""
    seq, mask = args
    rec = _run_case((seq, mask, [6.0], False))
    return [seq, rec["mask"] or "", rec["logz64"], rec["mfe"], rec["mea"]["6.0"], rec["post_sha256"][:16]]


def exhaustive_cases():
    cases = []
    for L in range(1, 6):
        for t in itertools.product("ACGU", repeat=L):
            cases.append(("".join(t), None))
    for L in range(1, 5):
        for t in itertools.product("ACGU", repeat=L):
            for m in itertools.product((0, 1), repeat=L):
                if any(m):
                    cases.append(("".join(t), list(m)))
    return cases


def long_cases():
    rng = np.random.default_rng(20261203)
    out = []
    for L, p, alpha in ((300, 0.1, "ACGU"), (350, 0.0, "ACGU"), (400, 0.1, "ACGU"), (450, 0.3, "ACGUN"),
                        (500, 0.1, "ACGU"), (600, 0.1, "ACGU"), (600, 0.0, "ACGU")):
        seq = rand_seq(rng, L, alpha)
        mask = (rng.random(L) < p).astype(np.int8).tolist() if p > 0 else None
        out.append((seq, mask, [6.0], False))
    return out


def xlong_cases():
    rng = np.random.default_rng(20261204)
    s800 = rand_seq(rng, 800)
    s1000 = rand_seq(rng, 1000)
    m1000 = (rng.random(1000) < 0.1).astype(np.int8).tolist()
    return [(s800, None, [6.0], False), (s1000, m1000, [6.0], False)]


def rand_seq(rng, L, alphabet="ACGU"):
    return "".join(rng.choice(np.array(list(alphabet)), size=L))


def build_cases():
    cases = []
    gam = [6.0]
    gam_multi = [0.5, 1.0, 2.0, 4.0, 6.0, 8.0, 16.0]
    # reference literal known answer (README.md:101,104)
    cases.append(("GGGGAAAACCCC", None, gam_multi, True))
    cases.append(("GCGCGCAAAAGCGCGCAAAAGCGC", None, gam_multi, True))
    # edge cases: empty, tiny, non-ACGU, lowercase, T
    for seq in ["", "A", "GC", "GAC", "GGGAAAUCC", "NNNNGGGGAAAACCCCNNNN", "ggggaaaacccc",
                "GGGGTTTTCCCCAAAA", "ACGUXACGU-ACGU"]:
        cases.append((seq, None, gam, True))
    cases.append(("GGGGAAAACCCC", [0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0], gam, True))
    cases.append(("GGGGAAAACCCC", [1] * 12, gam, True))
    rng = np.random.default_rng(20260101)
    # small random: lengths 4..60, half masked (Bernoulli 0.1 / 0.3), some N
    for t in range(200):
        L = int(rng.integers(4, 61))
        alpha = "ACGU" if t % 7 else "ACGUN"
        seq = rand_seq(rng, L, alpha)
        mask = None
        if t % 2 == 1:
            p = 0.1 if t % 4 == 1 else 0.3
            mask = (rng.random(L) < p).astype(np.int8).tolist()
        cases.append((seq, mask, gam_multi if t % 10 == 0 else gam, t < 40))
    # medium: 128 nt unmasked, 200 nt with Bernoulli(0.1) mask
    for t in range(6):
        cases.append((rand_seq(rng, 128), None, gam, False))
    for t in range(4):
        L = 200
        seq = rand_seq(rng, L)
        mask = (rng.random(L) < 0.1).astype(np.int8).tolist()
        cases.append((seq, mask, [6.0, 2.0], False))
    return cases


def validation_script_sequences():
    """Sequences drawn exactly as tests/test_validation.py:15-27 and :67-69 draw them."""
    rng = np.random.default_rng(0)
    bases = np.array(list("ACGU"))
    seqs = ["".join(rng.choice(bases, size=int(rng.integers(30, 129)))) for _ in range(60)]
    # check [4]: L=24 sequence and its Bernoulli(0.3) forced-unpaired mask
    s4 = "".join(rng.choice(bases, size=24))
    m4 = (rng.random(24) < 0.3).astype(np.int8).tolist()
    return seqs, s4, m4


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--ref", required=True, help="checkout of the reference (the directory holding gpu_contrafold/)")
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=None)
    ap.add_argument("--exhaustive", action="store_true", help="all short sequences (and masks): exhaustive.json.gz")
    ap.add_argument("--long", action="store_true", help="seven 300-600 nt sequences: long.json")
    ap.add_argument("--xlong", action="store_true", help="800 and 1,000 nt sequences: xlong.json")
    ap.add_argument("--mea200", type=int, default=0, metavar="N",
                    help="the first N sequences of the 200-nt MEA workload: mea200_subset.json.gz")
    args = ap.parse_args()
    if args.mea200:
        sys.path.insert(0, REPO)
        from contrafold_gpu_gb300 import workloads
        sb, mask = workloads.mea_200()
        seqs = workloads.as_strings(sb)[:args.mea200]
        masks = [m.astype(np.int8).tolist() for m in mask[:args.mea200]]
        t0 = time.time()
        with mp.get_context("spawn").Pool(args.jobs, initializer=_init, initargs=(args.ref,)) as pool:
            rows = pool.map(_run_small, list(zip(seqs, masks)), chunksize=4)
        out = args.out or os.path.join(HERE, "mea200_subset.json.gz")
        doc = {"generator": f"tests/golden/make_golden.py --mea200 {args.mea200}",
               "reference": "gpu_contrafold/cpu.py (pure Python under an identity numba.njit)",
               "workload": "contrafold_gpu_gb300.workloads.mea_200(): first sequences, in order",
               "seqs_sha256": hashlib.sha256("".join(seqs).encode()).hexdigest(),
               "fields": ["seq", "mask", "logz64", "mfe", "mea_gamma6", "post_sha256_16"], "cases": rows}
        with gzip.open(out, "wt") as fh:
            json.dump(doc, fh, separators=(",", ":"))
        print(f"wrote {len(rows)} cases to {out} in {time.time() - t0:.0f}s")
        return
    if args.long or args.xlong:
        cases = long_cases() if args.long else xlong_cases()
        t0 = time.time()
        with mp.get_context("spawn").Pool(min(args.jobs, len(cases)), initializer=_init, initargs=(args.ref,)) as pool:
            order = sorted(range(len(cases)), key=lambda k: -len(cases[k][0]))
            res = pool.map(_run_case, [cases[k] for k in order], chunksize=1)
        recs = [None] * len(cases)
        for k, r in zip(order, res):
            recs[k] = r
        out = args.out or os.path.join(HERE, "long.json" if args.long else "xlong.json")
        with open(out, "w") as fh:
            json.dump({"generator": "tests/golden/make_golden.py " + ("--long" if args.long else "--xlong"),
                       "reference": "gpu_contrafold/cpu.py (pure Python under an identity numba.njit)",
                       "cases": recs}, fh, indent=0)
        print(f"wrote {len(recs)} cases to {out} in {time.time() - t0:.0f}s")
        return
    if args.exhaustive:
        cases = exhaustive_cases()
        t0 = time.time()
        with mp.get_context("spawn").Pool(args.jobs, initializer=_init, initargs=(args.ref,)) as pool:
            rows = pool.map(_run_small, cases, chunksize=64)
        out = args.out or os.path.join(HERE, "exhaustive.json.gz")
        doc = {"generator": "tests/golden/make_golden.py --exhaustive",
               "reference": "gpu_contrafold/cpu.py (pure Python under an identity numba.njit)",
               "fields": ["seq", "mask", "logz64", "mfe", "mea_gamma6", "post_sha256_16"], "cases": rows}
        with gzip.open(out, "wt") as fh:
            json.dump(doc, fh, separators=(",", ":"))
        print(f"wrote {len(rows)} cases to {out} in {time.time() - t0:.0f}s")
        return
    args.out = args.out or os.path.join(HERE, "golden.json")

    R = load_reference(args.ref)
    P = R.load()
    sys.path.insert(0, REPO)
    from contrafold_gpu_gb300 import params as prm
    blob = prm.pack64(P)
    np.save(os.path.join(HERE, "params_blob64.npy"), blob)

    cases = build_cases()
    val_seqs, s4, m4 = validation_script_sequences()
    for sq in val_seqs[:20]:
        cases.append((sq, None, [6.0], False))
    cases.append((s4, m4, [6.0], True))

    ctx = mp.get_context("spawn")
    t0 = time.time()
    with ctx.Pool(args.jobs, initializer=_init, initargs=(args.ref,)) as pool:
        # longest first for load balance
        order = sorted(range(len(cases)), key=lambda k: -len(cases[k][0]))
        res = pool.map(_run_case, [cases[k] for k in order], chunksize=1)
    recs = [None] * len(cases)
    for k, r in zip(order, res):
        recs[k] = r
    out = {
        "generator": "tests/golden/make_golden.py",
        "reference": "gpu_contrafold/cpu.py (pure Python under an identity numba.njit)",
        "params_blob64_sha256": hashlib.sha256(blob.tobytes()).hexdigest(),
        "validation_script": {"seqs": val_seqs, "check4_seq": s4, "check4_mask": m4},
        "cases": recs,
    }
    with open(args.out, "w") as fh:
        json.dump(out, fh, indent=0)
    print(f"wrote {len(recs)} cases to {args.out} in {time.time() - t0:.0f}s")


if __name__ == "__main__":
    main()
