"""Fast_LogPlusEquals / Fast_Exp segment selection of the CUDA engine, restated in
float32 numpy with the constants parsed from its header (csrc/cf_device.cuh),
against the oracle's restatement of the reference (cpu.py:527-580, nested
comparisons) -- bitwise, on samples dense around every segment boundary, every
bin edge, the 11.86 cutoff and the zero threshold (-5e29).  CPU only.

What this pins: a unit-width bin of d (of -x for Fast_Exp) holds at most one
boundary, so (boundaries below the bin) + (d past the bin's boundary) picks the
reference's segment; and the engine's Fast_LogPlusEquals has no separate
zero-threshold test, which is exact for finite inputs (a smaller argument below
-5e29 either puts d past the cutoff or equals the larger one, and then adding
the cubic at 0 rounds back to it)."""
import os
import re

import numpy as np
import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "contrafold_gpu_gb300", "csrc", "cf_device.cuh")
f32 = np.float32


def _header():
    with open(HEADER) as fh:
        return fh.read()


def _define(src, name):
    return f32(float(re.search(r"#define %s \(\(float\)([-0-9.e]+)\)" % name, src).group(1)))


def _rows(block):
    rows = re.findall(r"\{\(float\)([-0-9.e]+), \(float\)([-0-9.e]+), \(float\)([-0-9.e]+), \(float\)([-0-9.e]+)\}",
                      block)
    return np.array(rows, dtype=np.float64).astype(f32)


@pytest.fixture(scope="module")
def consts():
    src = _header()
    lse_block = src[src.index("const float c[8][4]"):]
    lse_block = lse_block[:lse_block.index("t->lse[k]")]
    fexp_block = src[src.index("const float c[6][4]"):]
    fexp_block = fexp_block[:fexp_block.index("t->fexp[s]")]
    C = {
        "T": [_define(src, f"LSE_T{k}") for k in range(7)],
        "TMAX": _define(src, "LSE_TMAX"),
        "FT": [_define(src, f"FEXP_T{k}") for k in range(6)],
        "lse": _rows(lse_block),
        "fexp": _rows(fexp_block),
        "lse_bins": int(re.search(r"constexpr int kLseBins = (\d+);", src).group(1)),
        "fexp_bins": int(re.search(r"constexpr int kFexpBins = (\d+);", src).group(1)),
    }
    assert C["lse"].shape == (8, 4) and C["fexp"].shape == (6, 4)
    return C


def _cubic(c, x):
    r = f32(c[..., 0] * x)
    r = f32(r + c[..., 1])
    r = f32(r * x)
    r = f32(r + c[..., 2])
    r = f32(r * x)
    return f32(r + c[..., 3])


def _lse_bins(C):
    """load_poly_tables: per unit bin, boundaries below it and the one inside."""
    base, inner = [], []
    for b in range(C["lse_bins"]):
        lo, hi = f32(b), f32(b + 1)
        n, ins = 0, f32(3.402823466e38)
        for t in C["T"]:
            if t <= lo:
                n += 1
            elif t < hi:
                ins = t
        base.append(n)
        inner.append(ins)
    return np.array(base), np.array(inner, dtype=f32)


def _fexp_bins(C):
    base, inner = [], []
    U = [-t for t in C["FT"][1:]]
    for b in range(C["fexp_bins"]):
        lo, hi = f32(b), f32(b + 1)
        n, ins = 0, f32(-3.402823466e38)
        for u in U:
            if u >= hi:
                n += 1
            elif u >= lo:
                ins = u
        base.append(n)
        inner.append(ins)
    return np.array(base), np.array(inner, dtype=f32)


def engine_lse32(C, a, b):
    """cf_device.cuh lse32, elementwise in float32."""
    base, inner = _lse_bins(C)
    hi, lo = np.maximum(a, b), np.minimum(a, b)
    d = f32(hi - lo)
    binx = np.minimum(np.trunc(np.minimum(d, f32(2.0 ** 30))).astype(np.int64), C["lse_bins"] - 1)
    seg = base[binx] + (d >= inner[binx])
    with np.errstate(over="ignore", invalid="ignore"):   # huge d: the cubic overflows, the select drops it
        r = _cubic(C["lse"][seg], d)
        res = f32(lo + r)
    return np.where(d >= C["TMAX"], hi, res)


def engine_fexp32_neg(C, x):
    """cf_device.cuh fexp32 for x < 0, elementwise in float32."""
    base, inner = _fexp_bins(C)
    u = f32(-x)
    binx = np.minimum(np.trunc(np.minimum(u, f32(2.0 ** 30))).astype(np.int64), C["fexp_bins"] - 1)
    seg = base[binx] + (u <= inner[binx])
    r = _cubic(C["fexp"][seg], x)
    return np.where(x < C["FT"][0], f32(0.0), r)


def test_each_unit_bin_holds_at_most_one_boundary(consts):
    for ts in (consts["T"], [-t for t in consts["FT"][1:]]):
        bins = [int(np.floor(t)) for t in ts]
        assert len(set(bins)) == len(bins), bins
    assert consts["lse_bins"] * 1.0 >= float(consts["TMAX"])      # d beyond the bins is past the cutoff
    assert consts["fexp_bins"] * 1.0 >= -float(consts["FT"][0])   # u beyond the bins is below Fast_Exp's zero


def _near(v, n=8):
    """float32 values within n ulps of v."""
    out = [f32(v)]
    up = dn = f32(v)
    for _ in range(n):
        up = np.nextafter(up, f32(np.inf))
        dn = np.nextafter(dn, f32(-np.inf))
        out += [up, dn]
    return out


def test_lse32_matches_reference_bitwise(consts, oracle):
    rng = np.random.default_rng(0)
    L = oracle.lib()
    pairs = []
    # typical scores
    a = rng.uniform(-60, 60, 6000).astype(f32)
    pairs += list(zip(a, f32(a - rng.uniform(0, 14, 6000).astype(f32))))
    # d exactly at / around every boundary, bin edge and the cutoff (lo = 0: d = hi exactly)
    marks = list(consts["T"]) + [consts["TMAX"]] + [f32(k) for k in range(1, 13)]
    for t in marks:
        for v in _near(t):
            pairs += [(v, f32(0.0)), (f32(0.0), v), (f32(v + f32(-3.5)), f32(-3.5))]
    # the zero threshold: arguments at and below -5e29, equal or not
    low = [f32(-1e30), f32(-5e29), np.nextafter(f32(-5e29), f32(-np.inf)), f32(-6e29), f32(-2e30), f32(-4e30),
           f32(-1e30 + 3e23)]
    for x in low:
        for y in low + [f32(0.0), f32(-12.5), f32(7.25), f32(-5e29 + 1e23)]:
            pairs += [(x, y), (y, x)]
    A = np.array([p[0] for p in pairs], dtype=f32)
    B = np.array([p[1] for p in pairs], dtype=f32)
    got = engine_lse32(consts, A, B)
    want = np.array([L.oracle_lse32(float(x), float(y)) for x, y in zip(A, B)], dtype=f32)
    bad = np.nonzero(got.view(np.uint32) != want.view(np.uint32))[0]
    assert bad.size == 0, [(A[k], B[k], got[k], want[k]) for k in bad[:5]]


def test_fexp32_matches_reference_bitwise(consts, oracle):
    rng = np.random.default_rng(1)
    L = oracle.lib()
    xs = list(-rng.uniform(0, 12, 8000).astype(f32))
    for t in list(consts["FT"]) + [f32(-k) for k in range(1, 11)]:
        xs += [v for v in _near(t) if v < 0]
    X = np.array(xs, dtype=f32)
    got = engine_fexp32_neg(consts, X)
    want = np.array([L.oracle_fexp32(float(x)) for x in X], dtype=f32)
    bad = np.nonzero(got.view(np.uint32) != want.view(np.uint32))[0]
    assert bad.size == 0, [(X[k], got[k], want[k]) for k in bad[:5]]
