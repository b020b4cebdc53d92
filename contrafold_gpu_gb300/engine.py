"""ctypes binding of the CUDA engine (libcontrafold_gb300.so, include/contrafold_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is
usable, every call raises `EngineError`.
"""
from __future__ import annotations

import concurrent.futures as cfut
import ctypes
import os
import threading
from typing import List, Optional, Sequence

import numpy as np

from . import params as _params

HERE = os.path.dirname(os.path.abspath(__file__))
# CONTRAFOLD_GB300_LIB selects another build of the library (the checked one
# of build.py --check); the default is the in-tree release build
LIB_PATH = os.environ.get("CONTRAFOLD_GB300_LIB") or os.path.join(HERE, "libcontrafold_gb300.so")

CF_OK, CF_EINVAL, CF_ENOMEM, CF_ETIMEOUT, CF_ECUDA, CF_EDEVICE, CF_ECANCELLED = 0, 1, 2, 3, 4, 5, 6
CF_MAX_LEN = 32767
_STATUS = {1: "invalid argument", 2: "out of device memory / over budget", 3: "device wait timed out",
           4: "CUDA error", 5: "device-side limit", 6: "cancelled"}

# Exported symbols of include/contrafold_gb300.h
SYMBOLS = ("cf_engine_create", "cf_engine_destroy", "cf_engine_set_params", "cf_engine_set_budget",
           "cf_engine_set_mode", "cf_engine_set_schedule", "cf_engine_set_priority", "cf_engine_set_shared",
           "cf_engine_set_group", "cf_engine_load_tuning",
           "cf_engine_tuning_rows", "cf_engine_set_grad_checkpoint", "cf_grad_arena_bytes", "cf_last_error",
           "cf_version", "cf_logz", "cf_logz64", "cf_bpp",
           "cf_mea", "cf_mfe", "cf_sample", "cf_sample_seeded", "cf_sample_tasks", "cf_grad", "cf_plan_create", "cf_plan_destroy", "cf_plan_arena_bytes",
           "cf_plan_run", "cf_plan_status", "cf_plan_set_timing", "cf_plan_phase_ms", "cf_plan_launches",
           "cf_plan_group", "cf_plan_set_graph", "cf_plan_schedule", "cf_server_create", "cf_server_destroy", "cf_server_configure", "cf_server_pause",
           "cf_server_submit", "cf_server_wait", "cf_server_cancel", "cf_server_replay", "cf_server_stats",
           "cf_server_set_limits")
CF_JOB_LOGZ, CF_JOB_LOGZ64, CF_JOB_BPP, CF_JOB_MEA, CF_JOB_MFE = 0, 1, 2, 3, 4


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{_STATUS.get(code, code)}] {msg}")
        self.code = code


_lib = None
_lib_lock = threading.Lock()


def load_library(path: str = LIB_PATH):
    """dlopen the engine library (raises if it has not been built)."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise EngineError(CF_ECUDA, f"engine library not built: {path} (run contrafold_gpu_gb300.build.build())")
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        vp, u8p, i64p = ctypes.c_void_p, P(ctypes.c_uint8), P(ctypes.c_int64)
        f32p, f64p = P(ctypes.c_float), P(ctypes.c_double)
        L.cf_engine_create.argtypes = [f32p, f64p, ctypes.c_int, P(vp)]
        L.cf_engine_destroy.argtypes = [vp]
        L.cf_engine_set_params.argtypes = [vp, f32p, f64p]
        L.cf_engine_set_budget.argtypes = [vp, ctypes.c_size_t]
        L.cf_engine_set_mode.argtypes = [vp, ctypes.c_int]
        L.cf_engine_set_schedule.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.cf_engine_set_priority.argtypes = [vp, ctypes.c_int]
        L.cf_engine_set_shared.argtypes = [vp, ctypes.c_int]
        L.cf_engine_set_group.argtypes = [vp, ctypes.c_int]
        L.cf_engine_load_tuning.argtypes = [vp, ctypes.c_char_p]
        L.cf_engine_tuning_rows.argtypes = [vp]
        L.cf_engine_set_grad_checkpoint.argtypes = [vp, ctypes.c_int32]
        L.cf_engine_set_grad_checkpoint.restype = ctypes.c_int
        L.cf_grad_arena_bytes.argtypes = [ctypes.c_int32, ctypes.c_int32]
        L.cf_grad_arena_bytes.restype = ctypes.c_size_t
        L.cf_last_error.restype = ctypes.c_char_p
        L.cf_version.restype = ctypes.c_char_p
        L.cf_logz.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, f32p]
        L.cf_logz64.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, f64p]
        L.cf_bpp.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, i64p, f32p, f32p]
        L.cf_mea.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, ctypes.c_float, ctypes.c_char_p]
        L.cf_mfe.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, ctypes.c_char_p]
        L.cf_sample.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
                                ctypes.c_char_p]
        L.cf_sample_seeded.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, ctypes.c_int32, P(ctypes.c_uint64),
                                       ctypes.c_char_p]
        L.cf_sample_tasks.argtypes = [vp, u8p, i64p, u8p, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
                                      ctypes.c_char_p]
        L.cf_plan_create.argtypes = [vp, ctypes.c_int32, i64p, ctypes.c_int32, P(vp)]
        L.cf_plan_destroy.argtypes = [vp]
        L.cf_plan_arena_bytes.argtypes = [vp]
        L.cf_plan_arena_bytes.restype = ctypes.c_size_t
        L.cf_plan_run.argtypes = [vp, vp, vp, ctypes.c_float, vp, vp]
        L.cf_plan_status.argtypes = [vp]
        L.cf_plan_set_timing.argtypes = [vp, ctypes.c_int]
        L.cf_plan_phase_ms.argtypes = [vp, f32p, ctypes.c_int32]
        L.cf_plan_launches.argtypes = [vp]
        L.cf_plan_group.argtypes = [vp]
        L.cf_plan_set_graph.argtypes = [vp, ctypes.c_int]
        L.cf_plan_schedule.argtypes = [vp]
        L.cf_plan_schedule.restype = ctypes.c_char_p
        for name in ("cf_engine_create", "cf_engine_destroy", "cf_engine_set_params", "cf_engine_set_budget",
                     "cf_engine_set_mode", "cf_engine_set_schedule", "cf_engine_set_priority", "cf_engine_set_shared",
                     "cf_engine_set_group", "cf_engine_load_tuning", "cf_engine_tuning_rows", "cf_logz", "cf_logz64", "cf_bpp", "cf_mea", "cf_mfe", "cf_sample",
                     "cf_sample_seeded", "cf_sample_tasks", "cf_plan_create", "cf_plan_destroy", "cf_plan_run", "cf_plan_status", "cf_plan_set_timing",
                     "cf_plan_phase_ms", "cf_plan_launches", "cf_plan_group", "cf_plan_set_graph"):
            getattr(L, name).restype = ctypes.c_int
        _lib = L
        return L


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct)) if a is not None else None


def _text_buffer(n: int):
    """A zeroed host byte buffer of n bytes and the char* to pass (large
    buffers come as untouched zero pages, so zeroing costs nothing up front)."""
    arr = np.zeros(max(int(n), 1), np.uint8)
    return arr, ctypes.cast(arr.ctypes.data, ctypes.c_char_p)


def _text(arr: np.ndarray, n: int) -> str:
    """The first n bytes of `arr` as ASCII text (one copy)."""
    return str(memoryview(arr)[:int(n)], "ascii")


def _parallel_cast(x: np.ndarray, dtype: np.dtype) -> np.ndarray:
    """x.astype(dtype), in chunks on up to 16 threads."""
    out = np.empty(x.size, dtype)
    n = x.size
    k = max(1, min(16, os.cpu_count() or 1, n // (1 << 22)))
    if k == 1:
        np.copyto(out, x, casting="unsafe")
        return out
    edges = np.linspace(0, n, k + 1).astype(np.int64)
    with cfut.ThreadPoolExecutor(k) as ex:
        list(ex.map(lambda i: np.copyto(out[edges[i]:edges[i + 1]], x[edges[i]:edges[i + 1]], casting="unsafe"),
                    range(k)))
    return out


class Batch:
    """A batch of sequences packed for the C-ABI: ASCII bytes, int64 offsets,
    optional mask bytes (1 = forced unpaired).  Masks follow the reference:
    None means unconstrained, longer masks are truncated (gpu.py:494)."""

    def __init__(self, seqs: Sequence[str], masks: Optional[Sequence] = None):
        self.seqs = [str(s) for s in seqs]
        self.n = len(self.seqs)
        lens = np.fromiter((len(s) for s in self.seqs), np.int64, self.n)
        if self.n and lens.max() > CF_MAX_LEN:
            raise ValueError(f"sequence longer than {CF_MAX_LEN} nt")
        self.lens = lens
        self.offsets = np.zeros(self.n + 1, np.int64)
        np.cumsum(lens, out=self.offsets[1:])
        self.total = int(self.offsets[-1])
        self.buf = np.frombuffer("".join(self.seqs).encode("ascii", errors="replace"), np.uint8)
        if self.buf.size != self.total:      # non-ASCII characters: encode per character
            self.buf = np.array([ord(c) if ord(c) < 128 else ord("N") for c in "".join(self.seqs)], np.uint8)
        self.mask = None
        if masks is not None and any(m is not None for m in masks):
            if len(masks) != self.n:
                raise ValueError("one mask (or None) per sequence is required")
            # one concatenation of per-sequence views (a per-sequence copy into
            # a zeroed buffer cost 6x as much on 10,000 sequences)
            zero = np.zeros(int(lens.max()) if self.n else 0, np.uint8)
            parts = []
            for b, (m, L) in enumerate(zip(masks, lens.tolist())):
                if m is None:
                    parts.append(zero[:L])
                    continue
                arr = m if isinstance(m, np.ndarray) and m.ndim == 1 else np.asarray(m).reshape(-1)
                if arr.size < L:
                    raise ValueError(f"mask of sequence {b} is shorter ({arr.size}) than the sequence ({L})")
                parts.append(arr[:L])
            mk = np.concatenate(parts) if parts else np.zeros(0, np.uint8)
            mk = (mk != 0).view(np.uint8)
            self.mask = mk if mk.size else np.zeros(1, np.uint8)

    def split_strings(self, raw, per: int = 1) -> List[str]:
        s = raw.decode("ascii") if isinstance(raw, (bytes, bytearray)) else raw
        o = self.offsets.tolist()
        return [s[o[b] * per:o[b + 1] * per] for b in range(self.n)]


class Engine:
    """One device engine (parameters resident in HBM, a stream, a work arena)."""

    def __init__(self, P: dict, device: int = 0, mode: str = "batched"):
        self.lib = load_library()
        self._h = ctypes.c_void_p()
        b32, b64 = _params.pack32(P), _params.pack64(P)
        self._check(self.lib.cf_engine_create(_p(b32, ctypes.c_float), _p(b64, ctypes.c_double), int(device),
                                              ctypes.byref(self._h)))
        self.device = device
        self.set_mode(mode)
        self._lock = threading.Lock()

    def _check(self, rc):
        if rc != CF_OK:
            msg = self.lib.cf_last_error()
            raise EngineError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.cf_engine_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, P: dict):
        b32, b64 = _params.pack32(P), _params.pack64(P)
        self._check(self.lib.cf_engine_set_params(self._h, _p(b32, ctypes.c_float), _p(b64, ctypes.c_double)))

    def set_mode(self, mode: str):
        self._check(self.lib.cf_engine_set_mode(self._h, {"plain": 0, "batched": 1}[mode]))
        self.mode = mode

    def set_schedule(self, kind: str = "auto", ctas_per_sm: int = 0):
        """Batched-path schedule: 'auto', 'warp', 'cta' (persistent, + residency cap), 'group',
        'cluster' (each sequence folded by a thread-block cluster: latency of long sequences);
        'queue' is refused by the library (the queue schedule is disabled)."""
        self._check(self.lib.cf_engine_set_schedule(self._h, {"auto": 0, "warp": 1, "cta": 2, "group": 3,
                                                              "cluster": 4, "queue": 5}[kind],
                                                    int(ctas_per_sm)))

    def set_priority(self, high: bool):
        """Fold at the device's highest stream priority (True) or its default (False)."""
        self._check(self.lib.cf_engine_set_priority(self._h, int(bool(high))))

    def set_shared(self, on: bool):
        """The device is shared with other engines' launches: no 512-thread CTAs, no clusters."""
        self._check(self.lib.cf_engine_set_shared(self._h, int(bool(on))))

    def set_group(self, group: int = 0):
        """Sequences per CTA of the grouped kernels (<= 32; up to 64 accepted and capped); 0 = automatic."""
        self._check(self.lib.cf_engine_set_group(self._h, int(group)))

    def set_budget(self, nbytes: int):
        self._check(self.lib.cf_engine_set_budget(self._h, int(nbytes)))

    def load_tuning(self, path: Optional[str] = None):
        """Schedule table of the automatic batched path, as written by
        `autotune --write-table` (None restores the built-in table)."""
        self._check(self.lib.cf_engine_load_tuning(self._h, None if path is None else os.fsencode(path)))

    @property
    def tuning_rows(self) -> int:
        return int(self.lib.cf_engine_tuning_rows(self._h))

    def set_grad_checkpoint(self, every: int = 0):
        """cf_grad keeps the inside FM2 on every `every`-th diagonal and
        recomputes the rest (1: all kept; 0: automatic).  Results are bitwise
        the same for every spacing."""
        self._check(self.lib.cf_engine_set_grad_checkpoint(self._h, int(every)))

    # ---- batch entry points ----
    def _args(self, B: Batch):
        return (self._h, _p(B.buf, ctypes.c_uint8) if B.total else None, _p(B.offsets, ctypes.c_int64),
                _p(B.mask, ctypes.c_uint8), ctypes.c_int32(B.n))

    def logz(self, B: Batch) -> np.ndarray:
        out = np.zeros(max(B.n, 1), np.float32)
        with self._lock:
            self._check(self.lib.cf_logz(*self._args(B), _p(out, ctypes.c_float)))
        return out[:B.n]

    def logz64(self, B: Batch) -> np.ndarray:
        out = np.zeros(max(B.n, 1), np.float64)
        with self._lock:
            self._check(self.lib.cf_logz64(*self._args(B), _p(out, ctypes.c_double)))
        return out[:B.n]

    def bpp(self, B: Batch, dtype=np.float32):
        """Returns (list of (L, L) matrices, float32 logZ array).  The device
        computes float32; dtype=np.float64 widens on the host, on several
        threads (numpy releases the GIL in casts)."""
        sq = B.lens * B.lens
        po = np.zeros(B.n + 1, np.int64)
        np.cumsum(sq, out=po[1:])
        post = np.zeros(max(int(po[-1]), 1), np.float32)
        z = np.zeros(max(B.n, 1), np.float32)
        with self._lock:
            self._check(self.lib.cf_bpp(*self._args(B), _p(po, ctypes.c_int64), _p(post, ctypes.c_float),
                                        _p(z, ctypes.c_float)))
        if np.dtype(dtype) != np.float32:
            post = _parallel_cast(post, np.dtype(dtype))
        mats = [post[po[b]:po[b + 1]].reshape(int(B.lens[b]), int(B.lens[b])) for b in range(B.n)]
        return mats, z[:B.n]

    def mea(self, B: Batch, gamma: float = 6.0) -> List[str]:
        arr, out = _text_buffer(B.total)
        with self._lock:
            self._check(self.lib.cf_mea(*self._args(B), ctypes.c_float(float(np.float32(gamma))), out))
        return B.split_strings(_text(arr, B.total))

    def mfe(self, B: Batch) -> List[str]:
        arr, out = _text_buffer(B.total)
        with self._lock:
            self._check(self.lib.cf_mfe(*self._args(B), out))
        return B.split_strings(_text(arr, B.total))

    def sample(self, B: Batch, n_samples: int, seed: int = 0, seeds: Optional[Sequence[int]] = None) -> List[List[str]]:
        """Samples per sequence.  With `seeds` (one per sequence) sequence b draws
        what it draws alone with seed seeds[b] (cf_sample_seeded)."""
        if n_samples < 0:
            raise ValueError("n_samples must be >= 0")
        arr, out = _text_buffer(B.total * n_samples)
        with self._lock:
            if seeds is None:
                self._check(self.lib.cf_sample(*self._args(B), ctypes.c_int32(n_samples),
                                               ctypes.c_uint64(seed & 0xFFFFFFFFFFFFFFFF), out))
            else:
                sd = np.array([int(x) & 0xFFFFFFFFFFFFFFFF for x in seeds], np.uint64)
                if sd.size != B.n:
                    raise ValueError("one seed per sequence is required")
                self._check(self.lib.cf_sample_seeded(*self._args(B), ctypes.c_int32(n_samples),
                                                      _p(sd, ctypes.c_uint64), out))
        raw = _text(arr, B.total * n_samples)
        res = []
        offs, lens = B.offsets.tolist(), B.lens.tolist()
        for b in range(B.n):
            L = lens[b]
            if L == 0:
                res.append([""] * n_samples)
                continue
            base = offs[b] * n_samples
            chunk = raw[base:base + L * n_samples]   # this sequence's samples, one after another
            res.append([chunk[i:i + L] for i in range(0, L * n_samples, L)])
        return res

    def sample_tasks(self, B: Batch, chunk: int = 4096, seed: int = 0) -> List[str]:
        """One sample per task with the chunk / seed semantics of the
        reference's fold_tasks_gpu, all tasks in one submission (cf_sample_tasks)."""
        arr, out = _text_buffer(B.total)
        with self._lock:
            self._check(self.lib.cf_sample_tasks(*self._args(B), ctypes.c_int32(int(chunk)),
                                                 ctypes.c_uint64(seed & 0xFFFFFFFFFFFFFFFF), out))
        return B.split_strings(_text(arr, B.total))


def grad_arena_bytes(L: int, every: int = 0) -> int:
    """Device bytes cf_grad uses for one sequence of L nt."""
    return int(load_library().cf_grad_arena_bytes(int(L), int(every)))


class Plan:
    """A device-resident batch (cf_plan_*): fixed lengths, resident descriptors
    and arena; `run` launches kernels only, on the given CUDA stream."""

    def __init__(self, engine: "Engine", job: int, offsets: np.ndarray):
        self.engine = engine
        self.lib = engine.lib
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self.n = len(self.offsets) - 1
        self._h = ctypes.c_void_p()
        engine._check(self.lib.cf_plan_create(engine._h, int(job), _p(self.offsets, ctypes.c_int64),
                                              ctypes.c_int32(self.n), ctypes.byref(self._h)))

    @property
    def arena_bytes(self) -> int:
        return int(self.lib.cf_plan_arena_bytes(self._h))

    @property
    def group(self) -> int:
        return int(self.lib.cf_plan_group(self._h))

    @property
    def launches(self) -> int:
        return int(self.lib.cf_plan_launches(self._h))

    def run(self, d_seqs: int, d_mask: int, d_out: int, gamma: float = 6.0, stream: int = 0):
        """Device pointers (ints) in, asynchronous on `stream` (a cudaStream_t handle)."""
        self.engine._check(self.lib.cf_plan_run(self._h, ctypes.c_void_p(d_seqs or None),
                                                ctypes.c_void_p(d_mask or None),
                                                ctypes.c_float(float(np.float32(gamma))),
                                                ctypes.c_void_p(d_out), ctypes.c_void_p(stream or None)))

    def status(self):
        self.engine._check(self.lib.cf_plan_status(self._h))

    def set_timing(self, on: bool):
        self.engine._check(self.lib.cf_plan_set_timing(self._h, 1 if on else 0))

    @property
    def schedule(self) -> str:
        """'plain', 'warp', 'cta' or 'group'."""
        return self.lib.cf_plan_schedule(self._h).decode()

    def set_graph(self, on: bool):
        """Replay the plan's launches as one CUDA graph while run arguments repeat."""
        self.engine._check(self.lib.cf_plan_set_graph(self._h, 1 if on else 0))

    def phase_ms(self) -> np.ndarray:
        ms = np.zeros(4, np.float32)
        self.engine._check(self.lib.cf_plan_phase_ms(self._h, _p(ms, ctypes.c_float), 4))
        return ms

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.cf_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_engines = {}
_engines_lock = threading.Lock()


def engine_for(P: dict, device: int = 0) -> Engine:
    """The engine bound to parameter dict P (created on first use, cached in P)."""
    key = ("_engine", device)
    eng = P.get(key) if isinstance(P, dict) else None
    if eng is None:
        with _engines_lock:
            eng = P.get(key)
            if eng is None:
                eng = Engine(P, device)
                P[key] = eng
    return eng
