"""cf_mea_scratch -- MEA folding that allocates no device memory -- against
cf_mea, both through the C-ABI.

The file name sorts last, so in a full run these calls come after every other
GPU test has used the device and the shared engine; the tests pass alone too."""
import ctypes

import numpy as np
import pytest

from contrafold_gpu_gb300.engine import Batch, EngineError, _p, load_library

CF_OK, CF_EINVAL = 0, 1
SCRATCH_BYTES = 64 * 1024 * 1024


def _scratch_fn():
    lib = load_library()
    f = lib.cf_mea_scratch
    P = ctypes.POINTER
    f.argtypes = [ctypes.c_void_p, P(ctypes.c_uint8), P(ctypes.c_int64), P(ctypes.c_uint8), ctypes.c_int32,
                  ctypes.c_float, ctypes.c_char_p]
    f.restype = ctypes.c_int
    return lib, f


def _mea_scratch(engine, B: Batch, gamma: float = 6.0):
    lib, f = _scratch_fn()
    out = ctypes.create_string_buffer(max(B.total, 1))
    rc = f(engine._h, _p(B.buf, ctypes.c_uint8) if B.total else None, _p(B.offsets, ctypes.c_int64),
           _p(B.mask, ctypes.c_uint8), ctypes.c_int32(B.n), ctypes.c_float(gamma), out)
    if rc != CF_OK:
        raise EngineError(rc, lib.cf_last_error().decode())
    return B.split_strings(out.raw[:B.total])


def _batch(seed, n, lo, hi, masked):
    rng = np.random.default_rng(seed)
    lens = [0, 1, 4, 31, 32, 33] + [int(x) for x in rng.integers(lo, hi, n)]
    seqs = ["".join(rng.choice(list("ACGU"), size=L)) for L in lens]
    masks = None
    if masked:
        masks = [(rng.random(L) < 0.1).astype(np.int8) if b % 3 == 0 else None for b, L in enumerate(lens)]
    return Batch(seqs, masks)


@pytest.mark.gpu
def test_scratch_matches_cf_mea_on_consecutive_calls(engine):
    torch = pytest.importorskip("torch")
    A = _batch(11, 120, 20, 320, masked=True)
    Bb = _batch(12, 40, 5, 90, masked=False)     # smaller: stale scratch from the first call must not leak
    want_a = engine.mea(A, 6.0)
    want_b = engine.mea(Bb, 2.5)
    got_a = _mea_scratch(engine, A, 6.0)         # first call on the device: set-up
    assert got_a == want_a
    free0 = torch.cuda.mem_get_info(0)[0]
    got_b = _mea_scratch(engine, Bb, 2.5)
    got_a2 = _mea_scratch(engine, A, 6.0)
    free1 = torch.cuda.mem_get_info(0)[0]
    assert got_b == want_b
    assert got_a2 == want_a
    assert free1 == free0, "device memory changed across calls that should allocate nothing"


def _pad32(w):
    return (w + 31) & ~31


def _slot_bytes(L):
    """Bytes of one warp fold slot for a longest sequence of L nt: the float32
    fold arena of the kernels (csrc/cf_device.cuh arena32): seven triangular
    tables, five (L + 2)-vectors, the pair list and the traceback queue."""
    t = _pad32((L + 1) * (L + 2) // 2)
    v = _pad32(L + 2)
    plist = _pad32(L + 3) + _pad32((L + 1) * (L + 2) // 4 + 1)   # int32 offsets + int16 list
    return 4 * (7 * t + 5 * v + plist + _pad32(4 * L + 16))


def _scratch_limit(nbytes, n=1):
    """Longest sequence for which a batch of n sequences, nbytes nucleotides and
    no mask leaves room for one CTA (8 warps) of fold slots in the scratch
    (csrc/cf_noalloc.cu layout_for)."""
    up = lambda x: (x + 255) & ~255
    arena = 256 + up(8 * (n + 1)) + up(24 * n) + up(nbytes) + up(nbytes)
    L = 1
    while 8 * _slot_bytes(L + 1) <= SCRATCH_BYTES - arena:
        L += 1
    return L


@pytest.mark.gpu
def test_scratch_at_the_length_limit(engine):
    """One sequence just at the longest length whose 8 fold slots fit folds like
    cf_mea; one nucleotide more is rejected with CF_EINVAL."""
    lim = _scratch_limit(0)
    lim = _scratch_limit(lim)          # the sequence's own input and output bytes
    assert 700 <= lim <= 800, lim
    rng = np.random.default_rng(31)
    seq = "".join(rng.choice(list("ACGU"), size=lim))
    B = Batch([seq])
    assert _mea_scratch(engine, B) == engine.mea(B)
    lib, f = _scratch_fn()
    B1 = Batch([seq + "A"])
    out = ctypes.create_string_buffer(B1.total)
    rc = f(engine._h, _p(B1.buf, ctypes.c_uint8), _p(B1.offsets, ctypes.c_int64), None, 1, 6.0, out)
    assert rc == CF_EINVAL and b"scratch" in lib.cf_last_error()


@pytest.mark.gpu
def test_scratch_rejects_what_does_not_fit(engine):
    lib, f = _scratch_fn()
    # longest sequence too long for one CTA of fold slots
    B = Batch(["ACGU" * 200])
    out = ctypes.create_string_buffer(B.total)
    rc = f(engine._h, _p(B.buf, ctypes.c_uint8), _p(B.offsets, ctypes.c_int64), None, 1, 6.0, out)
    assert rc == CF_EINVAL and b"scratch" in lib.cf_last_error()
    # too many nucleotides: 2 bytes each (sequence + dot-bracket) exceed the scratch
    n, L = 360_000, 100
    buf = np.full(n * L, ord("A"), np.uint8)
    offs = np.arange(n + 1, dtype=np.int64) * L
    out = ctypes.create_string_buffer(n * L)
    rc = f(engine._h, _p(buf, ctypes.c_uint8), _p(offs, ctypes.c_int64), None, n, 6.0, out)
    assert rc == CF_EINVAL and b"scratch" in lib.cf_last_error()
    # the same argument errors as cf_mea
    B = Batch(["GGGAAACCC"])
    out = ctypes.create_string_buffer(B.total)
    assert f(engine._h, _p(B.buf, ctypes.c_uint8), _p(B.offsets, ctypes.c_int64), None, 1, 0.0, out) == CF_EINVAL
    assert f(None, _p(B.buf, ctypes.c_uint8), _p(B.offsets, ctypes.c_int64), None, 1, 6.0, out) == CF_EINVAL
    assert f(engine._h, None, None, None, 0, 6.0, None) == CF_OK
    # a batch that fits still folds after the rejections
    assert _mea_scratch(engine, B) == engine.mea(B)
