"""The first 512 sequences of the 10,000 x 200 nt MEA workload (bases
default_rng(0), Bernoulli(0.1) mask default_rng(1)) against the reference's
own cpu.py (tests/golden/mea200_subset.json.gz, made by
tests/golden/make_golden.py --mea200 512): the oracle on the CPU -- MEA
(gamma 6) and Viterbi structures identical, FP64 logZ to 1e-9, float32
posterior bitwise -- and the CUDA engine on the GPU -- structures identical,
posterior bitwise."""
import gzip
import hashlib
import json
import os

import numpy as np
import pytest

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mea200_subset.json.gz")


@pytest.fixture(scope="module")
def subset():
    from contrafold_gpu_gb300 import workloads
    with gzip.open(FIXTURE, "rt") as fh:
        doc = json.load(fh)
    rows = doc["cases"]
    sb, mask = workloads.mea_200()
    seqs = workloads.as_strings(sb)[:len(rows)]
    masks = [m.astype(np.int8) for m in mask[:len(rows)]]
    assert hashlib.sha256("".join(seqs).encode()).hexdigest() == doc["seqs_sha256"]
    assert [r[0] for r in rows] == seqs
    assert [r[1] for r in rows] == ["".join(str(int(x)) for x in m) for m in masks]
    return rows, seqs, masks


def _digest_full(POST):
    return hashlib.sha256(np.ascontiguousarray(POST, np.float32).tobytes()).hexdigest()[:16]


def test_fixture_is_the_workload_prefix(subset):
    rows, seqs, masks = subset
    assert len(rows) >= 500 and all(len(s) == 200 for s in seqs)


def test_oracle_matches_reference_on_workload(subset, P, oracle):
    rows, seqs, masks = subset
    cores = os.cpu_count() or 1
    assert oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0, threads=cores) == [r[4] for r in rows]
    assert oracle.batch(oracle.JOB_MFE, seqs, P, masks, threads=cores) == [r[3] for r in rows]
    z = oracle.batch(oracle.JOB_LOGZ64, seqs, P, masks, threads=cores)
    for r, v in zip(rows, z):
        assert abs(v - r[2]) <= 1e-9 * max(1.0, abs(r[2])), r[2:]
    for k in range(0, len(rows), 16):
        _, POST = oracle.posterior(seqs[k], P, masks[k])
        assert _digest_full(POST) == rows[k][5], k


@pytest.mark.gpu
def test_engine_matches_reference_on_workload(subset, engine):
    from contrafold_gpu_gb300.engine import Batch
    rows, seqs, masks = subset
    engine.set_mode("batched")
    engine.set_schedule("auto")
    B = Batch(seqs, masks)
    assert engine.mea(B, 6.0) == [r[4] for r in rows]
    assert engine.mfe(B) == [r[3] for r in rows]
    mats, _ = engine.bpp(B)
    for k, (m, r) in enumerate(zip(mats, rows)):
        full = np.zeros((202, 202), np.float32)
        full[1:201, 1:201] = m
        assert _digest_full(full) == r[5], k
