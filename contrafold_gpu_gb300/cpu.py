"""Single-sequence API of the reference's `gpu_contrafold.cpu` module.

The reference runs these on the CPU (gpu_contrafold/cpu.py); here every call
runs on the GPU engine with the reference's arithmetic, so results are the
same:

* ``load(path=None)``                         cpu.py:40-135
* ``logZ(seq, P)``          FP64 exact inside  cpu.py:282-287
* ``mfe(seq, P, forced=None)``                 cpu.py:505-519
* ``bpp(seq, P, forced=None)``                 cpu.py:926-929
* ``mea(seq, P, gamma=6.0, forced=None)``      cpu.py:932-941
* ``encode(seq)``, ``canon_mat()``             cpu.py:138-151
"""
from __future__ import annotations

import numpy as np

from .params import (C_MAX_SINGLE, D_BULGE, D_HAIRPIN, D_IASYM, D_IEXP, D_INTERNAL, D_ISYM,  # noqa: F401
                     DEFAULT_PARAMS, NBASE, load)
from .engine import Batch, engine_for

NEG = -1e30
HALF = -5e29
B = {"A": 0, "C": 1, "G": 2, "U": 3, "T": 3}
CANON = {(0, 3), (3, 0), (1, 2), (2, 1), (2, 3), (3, 2)}


def code(c: str) -> int:
    return B.get(c, 4)


def encode(seq: str):
    """1-based codes s[0..L+1] (N sentinels) and L."""
    L = len(seq)
    s = np.full(L + 2, 4, dtype=np.int64)
    for i, c in enumerate(seq.upper()):
        s[i + 1] = code(c)
    return s, L


def canon_mat():
    m = np.zeros((NBASE, NBASE), dtype=np.int64)
    for a, b in CANON:
        m[a, b] = 1
    return m


def _one(seq, forced):
    return Batch([seq], None if forced is None else [forced])


def logZ(seq: str, P: dict) -> float:
    """FP64 log partition function (exact log1p/exp), no constraint."""
    return float(engine_for(P).logz64(_one(seq, None))[0])


def mfe(seq: str, P: dict, forced=None) -> str:
    """Maximum-probability (Viterbi) structure as a dot-bracket string."""
    return engine_for(P).mfe(_one(seq, forced))[0]


def bpp(seq: str, P: dict, forced=None) -> np.ndarray:
    """Base-pair probability matrix (L x L upper triangle, 0-based), float64."""
    mats, _ = engine_for(P).bpp(_one(seq, forced))
    return mats[0].astype(np.float64)


def mea(seq: str, P: dict, gamma: float = 6.0, forced=None) -> str:
    """Maximum-expected-accuracy structure (CONTRAfold default decoding)."""
    return engine_for(P).mea(_one(seq, forced), gamma)[0]
