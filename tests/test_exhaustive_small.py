"""Every ACGU sequence of 1-5 nt, and every (sequence, forced-unpaired mask) pair
of 1-4 nt (5,704 cases), against the reference's own cpu.py
(tests/golden/exhaustive.json.gz, made by tests/golden/make_golden.py
--exhaustive): FP64 logZ to 1e-9, Viterbi and MEA (gamma 6) structures
identical, float32 posterior matrices bitwise (SHA-256 digest).  The oracle on
the CPU; the CUDA engine on every schedule on the GPU."""
import gzip
import hashlib
import os

import numpy as np
import pytest

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "exhaustive.json.gz")


@pytest.fixture(scope="module")
def small():
    import json
    with gzip.open(FIXTURE, "rt") as fh:
        doc = json.load(fh)
    rows = doc["cases"]
    seqs = [r[0] for r in rows]
    masks = [np.array([int(c) for c in r[1]], np.int8) if r[1] else None for r in rows]
    return rows, seqs, masks


def _digest(POST):
    return hashlib.sha256(np.ascontiguousarray(POST, np.float32).tobytes()).hexdigest()[:16]


def test_fixture_covers_every_short_case(small):
    rows, seqs, masks = small
    assert len(rows) == sum(4 ** L for L in range(1, 6)) + sum(4 ** L * (2 ** L - 1) for L in range(1, 5))
    assert len({(r[0], r[1]) for r in rows}) == len(rows)


def test_oracle_matches_reference_exhaustive(small, P, oracle):
    rows, seqs, masks = small
    assert oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0) == [r[4] for r in rows]
    assert oracle.batch(oracle.JOB_MFE, seqs, P, masks) == [r[3] for r in rows]
    z = oracle.batch(oracle.JOB_LOGZ64, seqs, P, masks)
    for r, v in zip(rows, z):
        assert abs(v - r[2]) <= 1e-9 * max(1.0, abs(r[2])), r
    for k in range(0, len(rows), 7):
        _, POST = oracle.posterior(seqs[k], P, masks[k])
        assert _digest(POST) == rows[k][5], rows[k]


@pytest.mark.gpu
@pytest.mark.parametrize("path", ["plain", "warp", "cta", "group", "cluster"])
def test_engine_matches_reference_exhaustive(small, engine, path):
    from contrafold_gpu_gb300.engine import Batch
    rows, seqs, masks = small
    if path == "plain":
        engine.set_mode("plain")
    else:
        engine.set_mode("batched")
        engine.set_schedule(path)
    try:
        B = Batch(seqs, masks)
        assert engine.mea(B, 6.0) == [r[4] for r in rows]
        mats, _ = engine.bpp(B)
        for r, M in zip(rows, mats):
            L = len(r[0])
            full = np.zeros((L + 2, L + 2), np.float32)
            full[1:L + 1, 1:L + 1] = M
            assert _digest(full) == r[5], r
        z = engine.logz64(B)
        for r, v in zip(rows, z):
            assert abs(v - r[2]) <= 1e-9 * max(1.0, abs(r[2])), r
        assert engine.mfe(B) == [r[3] for r in rows]
    finally:
        engine.set_mode("batched")
        engine.set_schedule("auto")
