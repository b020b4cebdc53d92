"""Gradients of logZ: expected feature counts and soft unpaired bonuses.

    from contrafold_gpu_gb300 import grad
    res = grad.logz_grad(seqs, theta=None, bonus=bonuses, masks=None)
    res.logz            # (n,) float32 logZ with the bonuses
    res.d_theta         # (n, 708) d logZ / d raw feature (file order, grad.feature_names())
    res.d_blob          # (n, 2577) d logZ / d tied table entry (expected uses, FP64)
    res.d_bonus         # list of (L_b,) float64: d logZ / d bonus_t = P(t unpaired)

    LogZ.apply(theta, bonus, seqs) -> torch tensor of logZ with autograd to theta
    (708 raw features) and to the per-position bonuses (n, Lmax) zero-padded.

The model is linear in its parameters inside the exponent, so
d logZ / d(table entry) is the expected number of uses of that entry, which
the GPU computes from the inside/outside tables (include/contrafold_gb300.h,
cf_grad).  Raw features reach the tables through the loader's tying
(gpu_contrafold/cpu.py:40-135), a linear map: the raw-feature gradient is the
table gradient times its Jacobian, computed here exactly by perturbing each
feature of the parameter file (the loader's key-set fallbacks stay fixed).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import params as prm
from .engine import Batch, Engine, _p, load_library

_JAC_CACHE: Dict[tuple, np.ndarray] = {}


def feature_names(path: Optional[str] = None) -> List[str]:
    """Raw feature names in parameter-file order."""
    return list(prm.read_raw(path).keys())


def raw_vector(path: Optional[str] = None) -> np.ndarray:
    return np.array(list(prm.read_raw(path).values()), np.float64)


def tables_from_vector(theta: Sequence[float], names: Sequence[str]) -> dict:
    """Tied tables (the `load` dict) from raw feature values in `names` order."""
    return prm.tables_from_raw(dict(zip(names, (float(x) for x in theta))))


def write_params(path: str, theta: Sequence[float], names: Optional[Sequence[str]] = None) -> None:
    """Write a CONTRAfold parameter file ("name value" lines) -- e.g. after a gradient step."""
    names = list(names) if names is not None else feature_names()
    with open(path, "w") as fh:
        for k, v in zip(names, theta):
            fh.write(f"{k} {float(v):.10g}\n")


def tying_jacobian(names: Optional[Sequence[str]] = None) -> np.ndarray:
    """J[e, f] = d blob[e] / d theta[f] (CF_BLOB_LEN x n_features), exact.

    The loader is linear in the feature values for a fixed set of present keys
    (the reversed-key fallbacks depend only on which keys exist), so column f is
    blob(theta + e_f) - blob(theta) at theta = 0 with every key present."""
    names = tuple(names) if names is not None else tuple(feature_names())
    J = _JAC_CACHE.get(names)
    if J is not None:
        return J
    zero = {k: 0.0 for k in names}
    base = prm.pack64(prm.tables_from_raw(zero))
    J = np.zeros((prm.BLOB_LEN, len(names)))
    for f, k in enumerate(names):
        zero[k] = 1.0
        J[:, f] = prm.pack64(prm.tables_from_raw(zero)) - base
        zero[k] = 0.0
    _JAC_CACHE[names] = J
    return J


@dataclass
class GradResult:
    logz: np.ndarray
    d_blob: np.ndarray
    d_theta: np.ndarray
    d_bonus: List[np.ndarray]


def _engine_for_theta(theta, names, device):
    P = tables_from_vector(theta, names)
    return Engine(P, device=device), P


def logz_grad(seqs: Sequence[str], theta=None, bonus=None, masks=None, names=None, device: int = 0,
              engine: Optional[Engine] = None) -> GradResult:
    """logZ and its gradients for a batch (see module docstring).

    theta: raw feature values in `names` order (default: the bundled model);
    bonus: per-sequence arrays of per-position unpaired bonuses (or None)."""
    names = list(names) if names is not None else feature_names()
    if theta is None:
        theta = raw_vector()
    own = engine is None
    eng = engine
    if eng is None:
        eng, _ = _engine_for_theta(theta, names, device)
    B = Batch(seqs, masks)
    bon = None
    if bonus is not None:
        bon = np.zeros(max(B.total, 1), np.float32)
        for b, u in enumerate(bonus):
            if u is None:
                continue
            L = int(B.lens[b])
            u = np.asarray(u, np.float32).reshape(-1)
            if u.size < L:
                raise ValueError(f"bonus of sequence {b} is shorter than the sequence")
            bon[B.offsets[b]:B.offsets[b] + L] = u[:L]
    lib = load_library()
    if not hasattr(lib.cf_grad, "_cf_typed"):
        P_ = ctypes.POINTER
        lib.cf_grad.argtypes = [ctypes.c_void_p, P_(ctypes.c_uint8), P_(ctypes.c_int64), P_(ctypes.c_uint8),
                                ctypes.c_int32, P_(ctypes.c_float), P_(ctypes.c_float), P_(ctypes.c_double),
                                P_(ctypes.c_double)]
        lib.cf_grad.restype = ctypes.c_int
        lib.cf_grad._cf_typed = True
    logz = np.zeros(max(B.n, 1), np.float32)
    counts = np.zeros((max(B.n, 1), prm.BLOB_LEN), np.float64)
    unp = np.zeros(max(B.total, 1), np.float64)
    with eng._lock:
        eng._check(lib.cf_grad(eng._h, _p(B.buf, ctypes.c_uint8) if B.total else None,
                               _p(B.offsets, ctypes.c_int64), _p(B.mask, ctypes.c_uint8), ctypes.c_int32(B.n),
                               _p(bon, ctypes.c_float), _p(logz, ctypes.c_float), _p(counts, ctypes.c_double),
                               _p(unp, ctypes.c_double)))
    if own:
        eng.close()
    J = tying_jacobian(names)
    counts = counts[:B.n]
    return GradResult(logz=logz[:B.n], d_blob=counts, d_theta=counts @ J,
                      d_bonus=[unp[B.offsets[b]:B.offsets[b + 1]].copy() for b in range(B.n)])


def _torch_function():
    import torch

    class LogZ(torch.autograd.Function):
        """logZ(theta, bonus) for a fixed batch of sequences.

        forward(theta (n_features,), bonus (n, Lmax) or None, seqs, masks=None)
        -> (n,) float32 logZ.  Gradients: d logZ_b / d theta = expected raw
        feature counts of sequence b; d logZ_b / d bonus[b, t] = P(t unpaired)."""

        @staticmethod
        def forward(ctx, theta, bonus, seqs, masks=None):
            th = theta.detach().double().cpu().numpy()
            bl = None
            if bonus is not None:
                bn = bonus.detach().float().cpu().numpy()
                bl = [bn[b, :len(s)] for b, s in enumerate(seqs)]
            res = logz_grad(seqs, th, bl, masks)
            ctx.d_theta = torch.from_numpy(res.d_theta)
            Lmax = max((len(s) for s in seqs), default=0)
            db = np.zeros((len(seqs), Lmax))
            for b, v in enumerate(res.d_bonus):
                db[b, :len(v)] = v
            ctx.d_bonus = torch.from_numpy(db)
            ctx.has_bonus = bonus is not None
            return torch.from_numpy(res.logz).to(theta.device)

        @staticmethod
        def backward(ctx, g):
            g64 = g.detach().double().cpu()
            gt = (g64[:, None] * ctx.d_theta).sum(0).to(torch.float64)
            gb = (g64[:, None] * ctx.d_bonus) if ctx.has_bonus else None
            return gt, gb, None, None

    return LogZ


def __getattr__(name):
    if name == "LogZ":
        return _torch_function()
    raise AttributeError(name)
