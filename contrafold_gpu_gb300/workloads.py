"""Seeded synthetic inputs of the five measured workloads.

One definition each, shared by the benchmark and the parity tests, so that a
test of "the 10,000 x 200 nt MEA workload" folds exactly the sequences the
benchmark times.  Every base is i.i.d. uniform over ACGU (GC fraction 0.5);
no dataset is involved.

  logz_128      1,000 x 128 nt, default_rng(0) codes, no mask
  mea_200       10,000 x 200 nt, default_rng(0) codes (int8 draws),
                forced-unpaired mask Bernoulli(0.1) from default_rng(1)
  sampling      4,096 sequences, lengths U{40..400} and bases from default_rng(2)
  grad_300      512 x 300 nt, default_rng(0) codes, soft unpaired bonuses
                N(0, 0.5) from default_rng(3) (float32)
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np

ALPHA = np.frombuffer(b"ACGU", np.uint8)


def logz_128(n: int = 1000, L: int = 128) -> np.ndarray:
    """(n, L) ASCII bytes."""
    return ALPHA[np.random.default_rng(0).integers(0, 4, (n, L))].astype(np.uint8)


def mea_200(n: int = 10000, L: int = 200, p_mask: float = 0.1) -> Tuple[np.ndarray, np.ndarray]:
    """(n, L) ASCII bytes and (n, L) uint8 mask (1 = forced unpaired)."""
    idx = np.random.default_rng(0).integers(0, 4, size=(n, L), dtype=np.int8)
    seq_bytes = ALPHA[idx]
    mask = (np.random.default_rng(1).random((n, L)) < p_mask).astype(np.uint8)
    return seq_bytes, mask


def sampling(n: int = 4096, lo: int = 40, hi: int = 400) -> List[str]:
    rng = np.random.default_rng(2)
    lens = rng.integers(lo, hi + 1, n)
    return [ALPHA[rng.integers(0, 4, int(L))].tobytes().decode() for L in lens]


def grad_300(n: int = 512, L: int = 300) -> Tuple[List[str], np.ndarray]:
    """Sequences and (n, L) float32 bonuses."""
    codes = np.random.default_rng(0).integers(0, 4, (n, L))
    seqs = [bytes(r).decode() for r in ALPHA[codes].astype(np.uint8)]
    bonus = np.random.default_rng(3).normal(0, 0.5, (n, L)).astype(np.float32)
    return seqs, bonus


def as_strings(seq_bytes: np.ndarray) -> List[str]:
    return [bytes(r).decode() for r in seq_bytes]
