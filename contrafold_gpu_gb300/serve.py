"""Serving loop: continuous batching of single-sequence fold requests.

    from contrafold_gpu_gb300 import load, serve
    with serve.Server(load(), workers=4) as srv:
        t = srv.submit(serve.Request("mea", "GGGGAAAACCCC"))
        srv.result(t)                      # '((((....))))'
        rep = srv.replay(requests, arrivals)   # open-loop: latency per request

The loop itself is native (include/contrafold_gb300.h, cf_server_*): worker
threads, one engine and stream each, take the queue with the oldest request
(queues keyed by op, gamma / sample count and length bucket), fold up to
`max_batch` requests of it as one batch and publish the results.  Only
`long_workers` workers take buckets above `long_len` nt, so long folds never
occupy every worker.  A result
equals the same request folded alone: logZ (cf_logz), MEA (cf_mea), samples
(cf_sample_seeded with the request's own seed).  `mixed_workload` builds the
seeded request stream of the serving measurement (Poisson arrivals, log-normal
lengths, a logZ / MEA / sampling mix, some masked requests).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Union

import numpy as np

from . import params as _params
from .engine import CF_ETIMEOUT, CF_OK, EngineError, _p, load_library

OPS = {"logz": 0, "mea": 1, "sample": 2}


class _CRequest(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("n_samples", ctypes.c_int32), ("gamma", ctypes.c_float),
                ("reserved", ctypes.c_int32), ("seed", ctypes.c_uint64)]


@dataclass
class Request:
    op: str                      # "logz" | "mea" | "sample"
    seq: str
    mask: Optional[Sequence[int]] = None
    gamma: float = 6.0
    n_samples: int = 10
    seed: int = 0

    def c(self) -> _CRequest:
        if self.op not in OPS:
            raise ValueError(f"unknown op {self.op!r}")
        return _CRequest(OPS[self.op], int(self.n_samples) if self.op == "sample" else 0,
                         float(np.float32(self.gamma)) if self.op == "mea" else 0.0, 0,
                         int(self.seed) & 0xFFFFFFFFFFFFFFFF)


Result = Union[float, str, List[str]]


@dataclass
class ReplayResult:
    latency_ms: np.ndarray
    status: np.ndarray
    results: List[Optional[Result]] = field(default_factory=list)


def _bind(L):
    if getattr(L, "_cf_server_typed", False):
        return L
    P = ctypes.POINTER
    vp, u8p, i64p = ctypes.c_void_p, P(ctypes.c_uint8), P(ctypes.c_int64)
    L.cf_server_create.argtypes = [P(ctypes.c_float), P(ctypes.c_double), ctypes.c_int, ctypes.c_int32, P(vp)]
    L.cf_server_destroy.argtypes = [vp]
    L.cf_server_configure.argtypes = [vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                      P(ctypes.c_int32), ctypes.c_int32]
    L.cf_server_pause.argtypes = [vp, ctypes.c_int32]
    L.cf_server_set_limits.argtypes = [vp, ctypes.c_double, ctypes.c_int64]
    L.cf_server_submit.argtypes = [vp, P(_CRequest), u8p, ctypes.c_int32, u8p, P(ctypes.c_int64)]
    L.cf_server_wait.argtypes = [vp, ctypes.c_int64, ctypes.c_int32, P(ctypes.c_float), ctypes.c_char_p,
                                 ctypes.c_int64]
    L.cf_server_cancel.argtypes = [vp, ctypes.c_int64]
    L.cf_server_replay.argtypes = [vp, ctypes.c_int32, P(ctypes.c_double), P(_CRequest), u8p, i64p, u8p, i64p,
                                   P(ctypes.c_float), ctypes.c_char_p, P(ctypes.c_double), P(ctypes.c_int32)]
    L.cf_server_stats.argtypes = [vp, P(ctypes.c_double), ctypes.c_int32]
    for name in ("cf_server_create", "cf_server_destroy", "cf_server_configure", "cf_server_pause", "cf_server_set_limits",
                 "cf_server_submit", "cf_server_wait", "cf_server_cancel", "cf_server_replay", "cf_server_stats"):
        getattr(L, name).restype = ctypes.c_int
    L._cf_server_typed = True
    return L


def _encode(seq: str) -> np.ndarray:
    b = np.frombuffer(seq.encode("ascii", errors="replace"), np.uint8)
    if b.size != len(seq):
        b = np.array([ord(c) if ord(c) < 128 else ord("N") for c in seq], np.uint8)
    return b


class Server:
    """A running serving loop on one device (see module docstring)."""

    def __init__(self, P: dict, device: int = 0, workers: int = 6, max_batch: int = 4096,
                 max_batch_nt: int = 1 << 20, long_len: int = 256, long_workers: int = 2,
                 edges: Sequence[int] = (96, 192, 256, 384, 640), max_batch_cost: float = 0.0,
                 max_batch_arena: int = 0):
        self.lib = _bind(load_library())
        b32, b64 = _params.pack32(P), _params.pack64(P)
        self._h = ctypes.c_void_p()
        self._check(self.lib.cf_server_create(_p(b32, ctypes.c_float), _p(b64, ctypes.c_double), int(device),
                                              int(workers), ctypes.byref(self._h)))
        self._meta = {}
        e = np.asarray(edges, np.int32)
        self._check(self.lib.cf_server_configure(self._h, int(max_batch), int(max_batch_nt), int(long_len),
                                                 int(min(long_workers, workers)), _p(e, ctypes.c_int32), int(e.size)))
        self.set_limits(max_batch_cost, max_batch_arena)

    def set_limits(self, max_batch_cost: float = 0.0, max_batch_arena: int = 0):
        """Cap a batch's predicted work (sum of L^3) and its device arena bytes (0 = no cap)."""
        self._check(self.lib.cf_server_set_limits(self._h, float(max_batch_cost), int(max_batch_arena)))

    def _check(self, rc):
        if rc != CF_OK:
            msg = self.lib.cf_last_error()
            raise EngineError(rc, msg.decode() if msg else "")

    def close(self):
        if self._h.value:
            self.lib.cf_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pause(self, on: bool = True):
        self._check(self.lib.cf_server_pause(self._h, 1 if on else 0))

    def submit(self, req: Request) -> int:
        s = _encode(req.seq)
        m = None
        if req.mask is not None:
            m = (np.asarray(req.mask).reshape(-1)[:s.size] != 0).astype(np.uint8)
            if m.size < s.size:
                raise ValueError("mask is shorter than the sequence")
        t = ctypes.c_int64()
        cr = req.c()
        self._check(self.lib.cf_server_submit(self._h, ctypes.byref(cr), _p(s, ctypes.c_uint8) if s.size else None,
                                              int(s.size), _p(m, ctypes.c_uint8), ctypes.byref(t)))
        self._meta[t.value] = (req.op, s.size, req.n_samples)
        return t.value

    def result(self, ticket: int, timeout: Optional[float] = None) -> Result:
        op, L, ns = self._meta[ticket]
        cap = max(L * (ns if op == "sample" else 1), 1)
        out = ctypes.create_string_buffer(cap)
        lz = ctypes.c_float()
        ms = -1 if timeout is None else int(timeout * 1000)
        rc = self.lib.cf_server_wait(self._h, ticket, ms, ctypes.byref(lz), out, cap)
        if rc != CF_ETIMEOUT:   # a timed-out request stays queued or running
            self._meta.pop(ticket, None)
        self._check(rc)
        return _unpack(op, L, ns, lz.value, out.raw)

    def cancel(self, ticket: int):
        self._check(self.lib.cf_server_cancel(self._h, ticket))

    def stats(self) -> dict:
        v = np.zeros(10)
        self._check(self.lib.cf_server_stats(self._h, _p(v, ctypes.c_double), 10))
        return dict(batches=int(v[0]), done=int(v[1]), nucleotides=int(v[2]), cancelled=int(v[3]),
                    busy_s=float(v[4]), queued=int(v[5]), wait_s=float(v[6]), max_wait_s=float(v[7]),
                    serve_s=float(v[8]), max_serve_s=float(v[9]))

    def replay(self, requests: Sequence[Request], arrivals: Sequence[float], keep_results: bool = True) -> ReplayResult:
        """Open-loop replay: request k is submitted arrivals[k] seconds after the
        start by the native replay loop, whatever the server's progress."""
        n = len(requests)
        t = np.ascontiguousarray(arrivals, np.float64)
        if t.size != n:
            raise ValueError("one arrival time per request")
        creq = (_CRequest * max(n, 1))(*[r.c() for r in requests])
        enc = [_encode(r.seq) for r in requests]
        lens = np.array([e.size for e in enc], np.int64)
        offs = np.zeros(n + 1, np.int64)
        np.cumsum(lens, out=offs[1:])
        buf = np.concatenate(enc) if n and offs[-1] else np.zeros(1, np.uint8)
        mask = None
        if any(r.mask is not None for r in requests):
            mask = np.zeros(max(int(offs[-1]), 1), np.uint8)
            for k, r in enumerate(requests):
                if r.mask is not None:
                    mask[offs[k]:offs[k + 1]] = np.asarray(r.mask).reshape(-1)[:lens[k]] != 0
        per = np.array([lens[k] * (r.n_samples if r.op == "sample" else (0 if r.op == "logz" else 1))
                        for k, r in enumerate(requests)], np.int64)
        oo = np.zeros(n + 1, np.int64)
        np.cumsum(per, out=oo[1:])
        out = ctypes.create_string_buffer(max(int(oo[-1]), 1))
        lz = np.zeros(max(n, 1), np.float32)
        lat = np.zeros(max(n, 1), np.float64)
        st = np.zeros(max(n, 1), np.int32)
        self._check(self.lib.cf_server_replay(self._h, n, _p(t, ctypes.c_double), creq, _p(buf, ctypes.c_uint8),
                                              _p(offs, ctypes.c_int64), _p(mask, ctypes.c_uint8),
                                              _p(oo, ctypes.c_int64), _p(lz, ctypes.c_float), out,
                                              _p(lat, ctypes.c_double), _p(st, ctypes.c_int32)))
        res = ReplayResult(latency_ms=lat[:n].copy(), status=st[:n].copy())
        if keep_results:
            raw = out.raw
            for k, r in enumerate(requests):
                if st[k] != CF_OK:
                    res.results.append(None)
                elif r.op == "logz":
                    res.results.append(float(lz[k]))
                else:
                    res.results.append(_unpack(r.op, int(lens[k]), r.n_samples, 0.0, raw[oo[k]:oo[k + 1]]))
        return res


def _unpack(op: str, L: int, ns: int, lz: float, raw: bytes) -> Result:
    if op == "logz":
        return float(lz)
    if op == "mea":
        return raw[:L].decode("ascii")
    s = raw[:L * ns].decode("ascii")
    return [s[i * L:(i + 1) * L] for i in range(ns)]


def mixed_workload(n: int, rate: float, seed: int = 0, median_len: float = 150.0, sigma: float = 0.6,
                   min_len: int = 30, max_len: int = 1000, mix=(0.4, 0.4, 0.2), mask_frac: float = 0.1,
                   mask_p: float = 0.1, gamma: float = 6.0, n_samples: int = 10):
    """Seeded open-loop request stream: Poisson arrivals at `rate` requests/s,
    lengths log-normal (median `median_len`, log-sd `sigma`) clipped to
    [min_len, max_len], uniform ACGU bases, ops logZ / MEA / sampling in the
    proportions `mix`, a fraction `mask_frac` of requests carrying a
    Bernoulli(`mask_p`) forced-unpaired mask.  Returns (requests, arrivals)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    arrivals = np.cumsum(gaps) - gaps[0]
    lens = np.clip(np.rint(np.exp(rng.normal(np.log(median_len), sigma, n))), min_len, max_len).astype(int)
    ops = rng.choice(3, size=n, p=np.asarray(mix) / np.sum(mix))
    masked = rng.random(n) < mask_frac
    reqs = []
    alpha = np.frombuffer(b"ACGU", np.uint8)
    for k in range(n):
        L = int(lens[k])
        seq = alpha[rng.integers(0, 4, L)].tobytes().decode()
        mask = (rng.random(L) < mask_p).astype(np.int8) if masked[k] else None
        op = ("logz", "mea", "sample")[ops[k]]
        reqs.append(Request(op, seq, mask, gamma=gamma, n_samples=n_samples, seed=int(rng.integers(0, 2**63))))
    return reqs, arrivals

