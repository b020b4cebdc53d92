"""TEST INFRASTRUCTURE ONLY -- ctypes front end of the C oracle (cf_oracle.c).

The oracle is a CPU restatement of the reference engine gpu_contrafold/cpu.py
(loop order and operation order kept so FP32 results compare bitwise).  Only
tests, the smoke check and the CPU-baseline leg of the benchmark use it; the
product never imports this module.

Functions mirror the reference's host wrappers:
  logz64(seq, P, forced)   -> cpu.inside via cpu.logZ   (cpu.py:165-287)
  bpp(seq, P, forced)      -> cpu.bpp                   (cpu.py:926-929)
  mea(seq, P, gamma, forced) -> cpu.mea                 (cpu.py:932-941)
  mfe(seq, P, forced)      -> cpu.mfe                   (cpu.py:505-519)
  bpp_exact(seq, P, forced) -> the same posterior in FP64 with exact log1p/exp (ours)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None

JOB_MEA, JOB_MFE, JOB_LOGZ64, JOB_LOGZ32 = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile liboracle.so with the recipe in oracle/Makefile."""
    srcs = [os.path.join(HERE, f) for f in ("cf_oracle.c", "cf_oracle_post.inc", "Makefile")]
    if force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(LIB_PATH) < os.path.getmtime(f) for f in srcs):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        i8p, f32p, f64p, i64p = P(ctypes.c_int8), P(ctypes.c_float), P(ctypes.c_double), P(ctypes.c_int64)
        L.oracle_inside64.restype = ctypes.c_double
        L.oracle_inside64.argtypes = [i8p, ctypes.c_int, i8p, f64p, f64p]
        L.oracle_viterbi64.restype = None
        L.oracle_viterbi64.argtypes = [i8p, ctypes.c_int, i8p, f64p, i64p]
        L.oracle_posterior32.restype = ctypes.c_float
        L.oracle_posterior32.argtypes = [i8p, ctypes.c_int, i8p, f32p, f32p, f32p]
        L.oracle_posterior64x.restype = ctypes.c_double
        L.oracle_posterior64x.argtypes = [i8p, ctypes.c_int, i8p, f64p, f64p, f64p]
        L.oracle_posterior32_tabs_len.restype = ctypes.c_size_t
        L.oracle_posterior32_tabs_len.argtypes = [ctypes.c_int]
        L.oracle_mea_decode32.restype = None
        L.oracle_mea_decode32.argtypes = [f32p, ctypes.c_int, i8p, i8p, ctypes.c_float, i64p]
        L.oracle_lse32.restype = ctypes.c_float
        L.oracle_lse32.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_fexp32.restype = ctypes.c_float
        L.oracle_fexp32.argtypes = [ctypes.c_float]
        L.oracle_inside64_bonus.restype = ctypes.c_double
        L.oracle_inside64_bonus.argtypes = [i8p, ctypes.c_int, i8p, f64p, f64p]
        L.oracle_count_mea_ops.restype = None
        L.oracle_count_mea_ops.argtypes = [i8p, ctypes.c_int, i8p, f32p, ctypes.c_float, i64p]
        u8p = P(ctypes.c_uint8)
        L.oracle_batch.restype = ctypes.c_int
        L.oracle_batch.argtypes = [ctypes.c_int, u8p, i64p, u8p, ctypes.c_int, f32p, f64p,
                                   ctypes.c_float, ctypes.c_char_p, f64p, ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


_CODE = {"A": 0, "C": 1, "G": 2, "U": 3, "T": 3}


def encode(seq: str, forced=None):
    """1-based codes with N sentinels and the forced array (cpu.py:138-144, 505-511)."""
    L = len(seq)
    s = np.full(L + 2, 4, np.int8)
    for t, c in enumerate(seq.upper()):
        s[t + 1] = _CODE.get(c, 4)
    fo = np.zeros(L + 2, np.int8)
    if forced is not None:
        fo[1:L + 1] = np.asarray(forced, dtype=np.int64)[:L].astype(np.int8)
    return s, fo, L


def _blobs(P):
    from contrafold_gpu_gb300 import params as prm   # layout only
    b32 = P.get("_blob32")
    if b32 is None:
        b32 = P["_blob32"] = prm.pack32(P)
        P["_blob64"] = prm.pack64(P)
    return P["_blob32"], P["_blob64"]


def logz64(seq, P, forced=None) -> float:
    s, fo, L = encode(seq, forced)
    _, b64 = _blobs(P)
    return float(lib().oracle_inside64(_ptr(s, ctypes.c_int8), L, _ptr(fo, ctypes.c_int8),
                                       _ptr(b64, ctypes.c_double), None))


def logz64_bonus(seq, P, bonus=None, forced=None, blob64=None) -> float:
    """FP64 logZ with a per-position unpaired bonus (our extension of cpu.py:165-275;
    the reference has no bonus).  `blob64` overrides the parameter blob."""
    s, fo, L = encode(seq, forced)
    b64 = blob64 if blob64 is not None else _blobs(P)[1]
    u = None
    if bonus is not None:
        u = np.zeros(L + 2, np.float64)
        u[1:L + 1] = np.asarray(bonus, np.float64)[:L]
    return float(lib().oracle_inside64_bonus(_ptr(s, ctypes.c_int8), L, _ptr(fo, ctypes.c_int8),
                                             _ptr(np.ascontiguousarray(b64, np.float64), ctypes.c_double),
                                             _ptr(u, ctypes.c_double) if u is not None else None))


def inside64_tables(seq, P, forced=None):
    s, fo, L = encode(seq, forced)
    _, b64 = _blobs(P)
    n = L + 2
    tabs = np.empty(3 * n * n + n, np.float64)
    z = lib().oracle_inside64(_ptr(s, ctypes.c_int8), L, _ptr(fo, ctypes.c_int8),
                              _ptr(b64, ctypes.c_double), _ptr(tabs, ctypes.c_double))
    return z, tabs


def posterior(seq, P, forced=None, with_tables=False):
    """Returns (Z, POST[(L+2),(L+2)] float32[, dict of tables])."""
    s, fo, L = encode(seq, forced)
    b32, _ = _blobs(P)
    n = L + 2
    POST = np.empty((n, n), np.float32)
    tabs = None
    if with_tables:
        tabs = np.empty(lib().oracle_posterior32_tabs_len(L), np.float32)
    z = lib().oracle_posterior32(_ptr(s, ctypes.c_int8), L, _ptr(fo, ctypes.c_int8),
                                 _ptr(b32, ctypes.c_float), _ptr(POST, ctypes.c_float),
                                 _ptr(tabs, ctypes.c_float) if tabs is not None else None)
    if not with_tables:
        return np.float32(z), POST
    nn = n * n
    names = ["FC", "FM", "FM1", "FCo", "FMo", "FM1o", "POST"]
    d = {k: tabs[t * nn:(t + 1) * nn].reshape(n, n) for t, k in enumerate(names)}
    d["F5"] = tabs[7 * nn:7 * nn + n]
    d["F5o"] = tabs[7 * nn + n:7 * nn + 2 * n]
    return np.float32(z), POST, d


def bpp(seq, P, forced=None) -> np.ndarray:
    _, POST = posterior(seq, P, forced)
    L = len(seq)
    return POST[1:L + 1, 1:L + 1].astype(np.float64)


def bpp_exact(seq, P, forced=None) -> np.ndarray:
    """Exact Boltzmann pair probabilities: the posterior recurrences of
    cpu.py:583-820 in float64 with exact log1p/exp (ours; the reference's
    posterior is the float32 Fast_LogPlusEquals / Fast_Exp one, 1-6 % off the
    exact probabilities).  The sampler draws from this distribution."""
    s, fo, L = encode(seq, forced)
    _, b64 = _blobs(P)
    n = L + 2
    POST = np.empty((n, n), np.float64)
    lib().oracle_posterior64x(_ptr(s, ctypes.c_int8), L, _ptr(fo, ctypes.c_int8), _ptr(b64, ctypes.c_double),
                              _ptr(POST, ctypes.c_double), None)
    return POST[1:L + 1, 1:L + 1].copy()


def _db(pair, L):
    ch = ["."] * L
    for t in range(1, L + 1):
        if pair[t] > t:
            ch[t - 1] = "("
            ch[pair[t] - 1] = ")"
    return "".join(ch)


def mea(seq, P, gamma=6.0, forced=None) -> str:
    s, fo, L = encode(seq, forced)
    _, POST = posterior(seq, P, forced)
    pair = np.empty(L + 2, np.int64)
    lib().oracle_mea_decode32(_ptr(POST, ctypes.c_float), L, _ptr(fo, ctypes.c_int8),
                              _ptr(s, ctypes.c_int8), float(np.float32(gamma)),
                              _ptr(pair, ctypes.c_int64))
    return _db(pair, L)


def mfe(seq, P, forced=None) -> str:
    s, fo, L = encode(seq, forced)
    _, b64 = _blobs(P)
    pair = np.empty(L + 2, np.int64)
    lib().oracle_viterbi64(_ptr(s, ctypes.c_int8), L, _ptr(fo, ctypes.c_int8),
                           _ptr(b64, ctypes.c_double), _ptr(pair, ctypes.c_int64))
    return _db(pair, L)


def pack_batch(seqs, masks=None):
    """ASCII bytes + int64 offsets (+ optional mask bytes) for a list of sequences."""
    lens = np.array([len(s) for s in seqs], np.int64)
    offs = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum(lens, out=offs[1:])
    buf = np.frombuffer("".join(seqs).encode("ascii"), np.uint8).copy()
    mk = None
    if masks is not None and any(m is not None for m in masks):
        mk = np.zeros(int(offs[-1]), np.uint8)
        for b, m in enumerate(masks):
            if m is not None:
                L = int(lens[b])
                mk[offs[b]:offs[b] + L] = (np.asarray(m)[:L] != 0)
    return buf, offs, mk


def batch(job, seqs, P, masks=None, gamma=6.0, threads=None):
    """Run the oracle over a batch on `threads` host threads.  Returns
    structures (JOB_MEA / JOB_MFE) or logZ values (JOB_LOGZ64 / JOB_LOGZ32)."""
    b32, b64 = _blobs(P)
    buf, offs, mk = pack_batch(seqs, masks)
    n = len(seqs)
    out_s = ctypes.create_string_buffer(max(1, int(offs[-1])))
    out_z = np.zeros(max(1, n), np.float64)
    u8 = ctypes.c_uint8
    lib().oracle_batch(job, _ptr(buf, u8) if buf.size else None, _ptr(offs, ctypes.c_int64),
                       _ptr(mk, u8) if mk is not None else None, n,
                       _ptr(b32, ctypes.c_float), _ptr(b64, ctypes.c_double),
                       float(np.float32(gamma)), out_s, _ptr(out_z, ctypes.c_double),
                       int(threads or os.cpu_count() or 1))
    if job in (JOB_MEA, JOB_MFE):
        raw = out_s.raw[:int(offs[-1])].decode("ascii")
        return [raw[offs[b]:offs[b + 1]] for b in range(n)]
    return [float(z) for z in out_z[:n]]


# Cost, in FP32 operations, of one guarded update of each counter category
# (oracle_count_mea_ops), the cost model of the fold's roofline: single-branch
# LSE = 4 adds for the loop score + 1 for jB2 + 1 add of the inner value + 8 for
# Fast_LogPlusEquals (sub, 3 mul, 3 add, final add) = 14; bifurcation / other
# LSE = 1 add + 8 = 9; posterior Fast_Exp term = 8; MEA max-plus candidate = 1.
OP_COST = (14, 9, 9, 14, 9, 9, 8, 1)
# FP64 operations of the Viterbi forward pass per inside category (the same
# guarded candidates as the inside): single-branch = 5 adds + 1 compare,
# bifurcation = 1 add + 1 compare, other terms = 3 adds + 1 compare.
VITERBI_COST = (6, 2, 4)
COUNT_NAMES = ("inside_single", "inside_bif", "inside_other", "outside_single", "outside_bif",
               "outside_other", "posterior_terms", "mea_candidates")


def count_mea_ops(seq, P, forced=None, gamma=6.0):
    """Guarded-update counts of one MEA fold, per category (COUNT_NAMES)."""
    s, fo, L = encode(seq, forced)
    b32, _ = _blobs(P)
    cnt = np.zeros(8, np.int64)
    lib().oracle_count_mea_ops(_ptr(s, ctypes.c_int8), L, _ptr(fo, ctypes.c_int8), _ptr(b32, ctypes.c_float),
                               float(np.float32(gamma)), _ptr(cnt, ctypes.c_int64))
    return cnt
