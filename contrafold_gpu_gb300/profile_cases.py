"""Small, fixed cases of each kernel family for profiler captures.

    python -m contrafold_gpu_gb300.profile_cases <case>

Each case folds a seeded batch twice through the public engine (the second
launch is the one to capture, e.g. ``ncu -k regex:<kernel> -s 1 -c 1``), small
enough that a full-section capture ends in a minute or two:

  group    k_fold_group32<MEA>: 2,432 x 200 nt drawn as the MEA workload (10 % mask)
  viterbi  k_viterbi64: 1,216 x 200 nt drawn as the MEA workload
  sample   k_inside32acc + k_sample32: 1,024 sequences drawn as the sampling workload x 10 samples
  adj      k_adj_inside + k_adj_outside: 152 x 300 nt drawn as the gradient workload
"""
from __future__ import annotations

import sys


def run(case: str) -> None:
    from . import grad, load, workloads
    from .engine import Batch, Engine
    P = load()
    eng = Engine(P)
    sb, mask = workloads.mea_200(2432, 200)
    seqs, masks = workloads.as_strings(sb), list(mask)
    try:
        if case == "viterbi":
            B = Batch(seqs[:1216], masks[:1216])
            for _ in range(2):
                eng.mfe(B)
        elif case == "sample":
            B = Batch(workloads.sampling(1024))
            for _ in range(2):
                eng.sample(B, 10, seed=1)
        elif case == "adj":
            s4, bonus = workloads.grad_300(152, 300)
            for _ in range(2):
                grad.logz_grad(s4, None, list(bonus), engine=eng)
        elif case == "group":
            B = Batch(seqs, masks)
            for _ in range(2):
                eng.mea(B, 6.0)
        else:
            raise SystemExit(f"unknown case {case!r}: group, viterbi, sample or adj")
    finally:
        eng.close()


if __name__ == "__main__":
    run(sys.argv[1] if len(sys.argv) > 1 else "group")
    print("done")
