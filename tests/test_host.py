"""Host-side logic and the C-ABI library (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "contrafold_gb300.h")


def header_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*|void)\s+(cf_\w+)\s*\(", txt, re.M)))


def test_header_layout_matches_python(P):
    from contrafold_gpu_gb300 import params
    txt = open(HEADER).read()
    for name, key in [("BP", "bp"), ("STACK", "stack"), ("TM", "tm"), ("HC", "hc"), ("DL", "dl"),
                      ("DR", "dr"), ("HPCUM", "hp_cum"), ("CS", "cs"), ("I11", "i11"), ("B01", "b01"),
                      ("MB", "mb"), ("MU", "mu"), ("MP", "mp"), ("EU", "eu"), ("EP", "ep")]:
        m = re.search(rf"#define CF_OFF_{name}\s+(\d+)", txt)
        assert m and int(m.group(1)) == params.OFFSETS[key], name
    assert int(re.search(r"#define CF_BLOB_LEN\s+(\d+)", txt).group(1)) == params.BLOB_LEN


def test_library_builds_and_exports_every_symbol():
    from contrafold_gpu_gb300 import build, engine
    lib = build.build()
    syms = header_symbols()
    assert len(syms) >= 13
    L = ctypes.CDLL(lib)
    for s in syms:
        assert hasattr(L, s), s
    assert set(engine.SYMBOLS) <= set(syms)
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (cf_\w+)", out))
    assert set(syms) <= exported


def test_version_and_error_string_without_gpu():
    from contrafold_gpu_gb300 import engine
    L = engine.load_library()
    assert b"sm_103a" in L.cf_version()
    # invalid arguments are rejected on the host before any device work
    assert L.cf_engine_create(None, None, 0, None) == engine.CF_EINVAL
    assert b"NULL" in L.cf_last_error()
    assert L.cf_logz(None, None, None, None, 0, None) == engine.CF_EINVAL


def test_batch_packing_and_masks():
    from contrafold_gpu_gb300.engine import Batch
    B = Batch(["ACGU", "", "GGGAAAUCC"], [None, None, [1, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1]])
    assert B.offsets.tolist() == [0, 4, 4, 13]
    assert bytes(B.buf) == b"ACGUGGGAAAUCC"
    assert B.mask[4:13].tolist() == [1, 0, 0, 0, 0, 0, 0, 0, 1]   # longer masks are truncated
    assert B.split_strings(b"abcdefghijklm") == ["abcd", "", "efghijklm"]
    with pytest.raises(ValueError):
        Batch(["ACGU"], [[0, 1]])                                    # shorter mask -> error
    assert Batch(["AC"], [None]).mask is None


def test_batch_mask_types_match_per_sequence_packing():
    """Masks as lists, int8 / bool / uint8 arrays, 2-D rows and None, with
    nonzero values other than 1: the packed bytes equal a per-sequence copy
    of (mask != 0)."""
    from contrafold_gpu_gb300.engine import Batch
    rng = np.random.default_rng(5)
    lens = [int(x) for x in rng.integers(0, 40, 60)]
    seqs = ["".join(rng.choice(list("ACGU"), size=L)) for L in lens]
    masks = []
    for k, L in enumerate(lens):
        kind = k % 5
        m = rng.integers(0, 3, L + (k % 3))            # some masks longer than their sequence
        masks.append(None if kind == 0 else m.tolist() if kind == 1 else m.astype(np.int8) if kind == 2
                     else (m != 0) if kind == 3 else m.astype(np.uint8).reshape(1, -1))
    B = Batch(seqs, masks)
    want = np.zeros(max(sum(lens), 1), np.uint8)
    o = 0
    for m, L in zip(masks, lens):
        if m is not None:
            want[o:o + L] = np.asarray(m).reshape(-1)[:L] != 0
        o += L
    assert B.mask.dtype == np.uint8 and np.array_equal(B.mask[:sum(lens)], want[:sum(lens)])


def test_parallel_cast_equals_astype():
    from contrafold_gpu_gb300.engine import _parallel_cast
    rng = np.random.default_rng(6)
    for n in (0, 1, 5, (1 << 22) + 3, 3 * (1 << 22) + 17):
        x = rng.random(n, dtype=np.float32)
        y = _parallel_cast(x, np.dtype(np.float64))
        assert y.dtype == np.float64 and np.array_equal(y, x.astype(np.float64))


def test_params_loader_tying(P):
    from contrafold_gpu_gb300 import params
    raw = params.read_raw()
    assert len(raw) == 708
    # symmetric base pair and stacking fallback (cpu.py:51-64)
    assert P["bp"][0, 3] == P["bp"][3, 0] == raw["base_pair_AU"]
    assert P["bp"][4].sum() == 0 and P["stack"][4].sum() == 0
    # running sums
    assert np.isclose(P["hp_cum"][5], sum(raw[f"hairpin_length_at_least_{k}"] for k in range(6)))
    b32 = params.pack32(P)
    assert b32.dtype == np.float32 and b32.size == params.BLOB_LEN
    assert b32[params.OFFSETS["mu"]] == np.float32(P["mu"])


def test_checked_build_compiles_and_exports_every_symbol():
    """build.py --check: the same sources with per-subscript table checks
    (-DCF_CHECK) compile and export the whole C-ABI (no GPU needed)."""
    from contrafold_gpu_gb300 import build
    lib = build.build(check=True)
    assert lib.endswith("libcontrafold_gb300_check.so")
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    assert set(header_symbols()) <= set(re.findall(r" T (cf_\w+)", out))
