"""Batch API of the reference's `gpu_contrafold.gpu` module, on the GB300 engine.

Signatures and semantics follow gpu_contrafold/gpu.py:480-601:

* ``logZ_batch(seqs, P, forced_list=None, threads=128) -> list[float]``
* ``sample_batch(seqs, P, n_samples, forced_list=None, threads=128, seed=0)
  -> list[list[str]]``
* ``fold_tasks_gpu(seqs, forced_masks, P, chunk=4096, seed=0) -> list[str]``

`threads` is accepted for compatibility; the engine picks its own launch
shape.  Added batched forms of the single-sequence CPU calls of the
reference: ``mea_batch``, ``mfe_batch``, ``bpp_batch``, ``logZ64_batch``.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

from .engine import Batch, engine_for


def _masks(forced_list, n):
    if forced_list is None:
        return None
    if len(forced_list) != n:
        raise ValueError("forced_list must hold one entry (or None) per sequence")
    return list(forced_list)


def logZ_batch(seqs: Sequence[str], P: dict, forced_list=None, threads: int = 128) -> List[float]:
    """FP32 log partition function of every sequence (gpu.py:480-517)."""
    B = Batch(seqs, _masks(forced_list, len(seqs)))
    return [float(z) for z in engine_for(P).logz(B)]


def logZ64_batch(seqs: Sequence[str], P: dict, forced_list=None) -> List[float]:
    """FP64 log partition function with exact log1p/exp (cpu.py:165-275)."""
    B = Batch(seqs, _masks(forced_list, len(seqs)))
    return [float(z) for z in engine_for(P).logz64(B)]


def sample_batch(seqs: Sequence[str], P: dict, n_samples: int, forced_list=None, threads: int = 128,
                 seed: int = 0) -> List[List[str]]:
    """n_samples Boltzmann samples per sequence as dot-brackets (gpu.py:520-583)."""
    B = Batch(seqs, _masks(forced_list, len(seqs)))
    return engine_for(P).sample(B, int(n_samples), int(seed))


def fold_tasks_gpu(seqs: Sequence[str], forced_masks, P: dict, chunk: int = 4096, seed: int = 0) -> List[str]:
    """One Boltzmann sample per (sequence, mask) task (gpu.py:586-601).

    The samples are those of the reference's loop -- tasks sorted by length,
    chunks of `chunk`, chunk c0 sampled by sample_batch with seed + c0 -- but
    every task is folded in one device submission (cf_sample_tasks)."""
    if chunk <= 0:
        raise ValueError("chunk must be > 0")
    B = Batch(seqs, _masks(forced_masks, len(seqs)))
    return engine_for(P).sample_tasks(B, int(chunk), int(seed))


def fold_tasks_chunked(seqs: Sequence[str], forced_masks, P: dict, chunk: int = 4096, seed: int = 0) -> List[str]:
    """The reference's host loop for fold_tasks_gpu (one sample_batch call per
    chunk of the length-sorted tasks); fold_tasks_gpu returns the same samples."""
    n = len(seqs)
    out: List[Optional[str]] = [None] * n
    order = sorted(range(n), key=lambda k: len(seqs[k]))
    for c0 in range(0, n, chunk):
        idx = order[c0:c0 + chunk]
        sub = [seqs[k] for k in idx]
        fl = [forced_masks[k] for k in idx] if forced_masks is not None else None
        res = sample_batch(sub, P, 1, forced_list=fl, seed=seed + c0)
        for k, r in zip(idx, res):
            out[k] = r[0]
    return out  # type: ignore[return-value]


def mea_batch(seqs: Sequence[str], P: dict, gamma: float = 6.0, forced_list=None) -> List[str]:
    """MEA structures of a batch (cpu.py:932-941 semantics, all on the device)."""
    B = Batch(seqs, _masks(forced_list, len(seqs)))
    return engine_for(P).mea(B, gamma)


def mfe_batch(seqs: Sequence[str], P: dict, forced_list=None) -> List[str]:
    """Viterbi structures of a batch (cpu.py:505-519 semantics)."""
    B = Batch(seqs, _masks(forced_list, len(seqs)))
    return engine_for(P).mfe(B)


def bpp_batch(seqs: Sequence[str], P: dict, forced_list=None) -> List[np.ndarray]:
    """Base-pair probability matrices (float64, (L, L), upper triangle) of a batch."""
    B = Batch(seqs, _masks(forced_list, len(seqs)))
    mats, _ = engine_for(P).bpp(B, np.float64)
    return mats
