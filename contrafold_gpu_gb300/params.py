"""CONTRAfold complementary-model parameters: file parsing, feature tying, device packing.

`load(path)` returns the same dictionary the reference's loader returns
(gpu_contrafold/cpu.py:40-135): float64 tables keyed
``bp, stack, tm, hc, dl, dr, hp_cum, cs, i11, b01`` and float scalars
``mb, mu, mp, eu, ep``.  Index 4 of every base axis is the N/unknown code and
stays zero, so N never contributes a score.

The tying rules are the model's definition and therefore must agree with the
reference term by term:

* ``base_pair_XY`` / ``internal_1x1_nucleotides_XY`` are symmetric (either
  spelling of the key is accepted, cpu.py:51-55, 103-108);
* ``helix_stacking_abcd`` falls back to the reversed key ``dcba`` (cpu.py:57-64);
* the ``*_at_least_k`` families become running sums (cpu.py:85-95), summed
  left to right in float64;
* ``cs[l1, l2]`` -- the single-branch loop cost -- adds its parts in the
  order explicit, length, symmetric, asymmetry (cpu.py:114-130).  The order is
  kept because every later float32 table is a rounding of these float64 sums
  and bitwise parity of the posterior depends on it.

`pack32` / `pack64` flatten a parameter dictionary into the contiguous blob
the C-ABI takes (layout in include/contrafold_gb300.h, ``CF_OFF_*``).
"""
from __future__ import annotations

import os
from typing import Dict

import numpy as np

DEFAULT_PARAMS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                              "contrafold.params.complementary")

BASES = "ACGU"
CODE = {"A": 0, "C": 1, "G": 2, "U": 3, "T": 3}
NBASE = 5
C_MAX_SINGLE = 30
D_HAIRPIN = 30
D_BULGE = 30
D_INTERNAL = 30
D_ISYM = 15
D_IASYM = 28
D_IEXP = 4

# Flat blob layout shared with the C-ABI (include/contrafold_gb300.h).
_LAYOUT = (("bp", 25), ("stack", 625), ("tm", 625), ("hc", 25), ("dl", 125), ("dr", 125),
           ("hp_cum", 31), ("cs", 961), ("i11", 25), ("b01", 5),
           ("mb", 1), ("mu", 1), ("mp", 1), ("eu", 1), ("ep", 1))
OFFSETS = {}
_o = 0
for _name, _size in _LAYOUT:
    OFFSETS[_name] = _o
    _o += _size
BLOB_LEN = _o          # 2577 entries
SCALARS = ("mb", "mu", "mp", "eu", "ep")
TABLES = ("bp", "stack", "tm", "hc", "dl", "dr", "hp_cum", "cs", "i11", "b01")


def read_raw(path: str | None = None) -> Dict[str, float]:
    """Parse a CONTRAfold parameter file into {feature_name: value} (two-token lines)."""
    raw: Dict[str, float] = {}
    with open(path or DEFAULT_PARAMS) as fh:
        for line in fh:
            tok = line.split()
            if len(tok) == 2:
                raw[tok[0]] = float(tok[1])
    return raw


def _running_sum(raw, prefix, dmax, first):
    """Cumulative `prefix_at_least_k` for k = first..dmax (entries below `first` are 0)."""
    step = np.zeros(dmax + 1)
    for k in range(first, dmax + 1):
        step[k] = raw.get(f"{prefix}_at_least_{k}", 0.0)
    return np.cumsum(step)


def tables_from_raw(raw: Dict[str, float]) -> dict:
    """Tie the raw feature values into the scoring tables (see module docstring)."""
    g = raw.get
    bp = np.zeros((NBASE, NBASE))
    i11 = np.zeros((NBASE, NBASE))
    hc = np.zeros((NBASE, NBASE))
    for x in BASES:
        for y in BASES:
            v = g(f"base_pair_{x}{y}", g(f"base_pair_{y}{x}", 0.0))
            bp[CODE[x], CODE[y]] = bp[CODE[y], CODE[x]] = v
            v = g(f"internal_1x1_nucleotides_{x}{y}", g(f"internal_1x1_nucleotides_{y}{x}", 0.0))
            i11[CODE[x], CODE[y]] = i11[CODE[y], CODE[x]] = v
            hc[CODE[x], CODE[y]] = g(f"helix_closing_{x}{y}", 0.0)

    stack = np.zeros((NBASE,) * 4)
    tm = np.zeros((NBASE,) * 4)
    dl = np.zeros((NBASE,) * 3)
    dr = np.zeros((NBASE,) * 3)
    for a in BASES:
        for b in BASES:
            for c in BASES:
                ia, ib, ic = CODE[a], CODE[b], CODE[c]
                dl[ia, ib, ic] = g(f"dangle_left_{a}{b}{c}", 0.0)
                dr[ia, ib, ic] = g(f"dangle_right_{a}{b}{c}", 0.0)
                for d in BASES:
                    idx = (ia, ib, ic, CODE[d])
                    stack[idx] = g(f"helix_stacking_{a}{b}{c}{d}", g(f"helix_stacking_{d}{c}{b}{a}", 0.0))
                    tm[idx] = g(f"terminal_mismatch_{a}{b}{c}{d}", 0.0)

    hp_cum = _running_sum(raw, "hairpin_length", D_HAIRPIN, 0)
    bulge_cum = _running_sum(raw, "bulge_length", D_BULGE, 1)
    il_cum = _running_sum(raw, "internal_length", D_INTERNAL, 2)
    isym_cum = _running_sum(raw, "internal_symmetric_length", D_ISYM, 1)
    iasym_cum = _running_sum(raw, "internal_asymmetry", D_IASYM, 1)

    iexp = np.zeros((D_IEXP + 1, D_IEXP + 1))
    for l1 in range(1, D_IEXP + 1):
        for l2 in range(1, D_IEXP + 1):
            iexp[l1, l2] = g(f"internal_explicit_{min(l1, l2)}_{max(l1, l2)}", 0.0)

    b01 = np.zeros(NBASE)
    for x in BASES:
        b01[CODE[x]] = g(f"bulge_0x1_nucleotides_{x}", 0.0)

    cs = np.zeros((C_MAX_SINGLE + 1, C_MAX_SINGLE + 1))
    for l1 in range(C_MAX_SINGLE + 1):
        for l2 in range(C_MAX_SINGLE + 1 - l1):
            if l1 == 0 and l2 == 0:
                continue
            if l1 == 0 or l2 == 0:                        # bulge
                cs[l1, l2] = bulge_cum[min(D_BULGE, l1 + l2)]
                continue
            acc = 0.0                                     # interior loop
            if l1 <= D_IEXP and l2 <= D_IEXP:
                acc += iexp[l1, l2]
            acc += il_cum[min(D_INTERNAL, l1 + l2)]
            if l1 == l2:
                acc += isym_cum[min(D_ISYM, l1)]
            acc += iasym_cum[min(D_IASYM, abs(l1 - l2))]
            cs[l1, l2] = acc

    return dict(bp=bp, stack=stack, tm=tm, hc=hc, dl=dl, dr=dr, hp_cum=hp_cum, cs=cs,
                i11=i11, b01=b01, mb=raw["multi_base"], mu=raw["multi_unpaired"],
                mp=raw["multi_paired"], eu=raw["external_unpaired"], ep=raw["external_paired"])


def load(path: str | None = None) -> dict:
    """Load a CONTRAfold parameter file (default: the bundled complementary model).

    Same keys, shapes and float64 values as gpu_contrafold.cpu.load
    (gpu_contrafold/cpu.py:40-135).
    """
    return tables_from_raw(read_raw(path))


def _pack(P: dict, dtype) -> np.ndarray:
    blob = np.zeros(BLOB_LEN, dtype=dtype)
    for name, size in _LAYOUT:
        o = OFFSETS[name]
        if name in SCALARS:
            blob[o] = dtype(P[name])
        else:
            arr = np.asarray(P[name], dtype=np.float64).reshape(-1)
            assert arr.size == size, (name, arr.size)
            blob[o:o + size] = arr.astype(dtype)   # float64 -> float32 rounding, as cpu.py:898-910
    return blob


def pack32(P: dict) -> np.ndarray:
    """float32 blob: every float64 table entry rounded once (gpu_contrafold/cpu.py:898-910)."""
    return _pack(P, np.float32)


def pack64(P: dict) -> np.ndarray:
    """float64 blob (for the FP64 inside and the Viterbi decoder)."""
    return _pack(P, np.float64)
