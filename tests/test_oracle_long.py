"""Pin the oracle at 300-1,000 nt to the reference itself (tests/golden/long.json
and xlong.json, made by tests/golden/make_golden.py --long / --xlong from
gpu_contrafold/cpu.py): FP64 logZ to 1e-9 relative, Viterbi and MEA structures
identical, float32 posterior matrices bitwise (SHA-256).  The GPU tests compare
the engine with the oracle at these lengths (600 nt, 600-1,000 nt on the
cluster schedule).  CPU only."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import mask_of

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as fh:
        return json.load(fh)["cases"]


@pytest.fixture(scope="module")
def long_cases():
    return _load("long.json")


def test_long_fixture_lengths(long_cases):
    assert sorted(len(c["seq"]) for c in long_cases) == [300, 350, 400, 450, 500, 600, 600]


def _check(cases, P, oracle):
    seqs = [c["seq"] for c in cases]
    masks = [mask_of(c) for c in cases]
    assert oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0) == [c["mea"]["6.0"] for c in cases]
    assert oracle.batch(oracle.JOB_MFE, seqs, P, masks) == [c["mfe"] for c in cases]
    z = oracle.batch(oracle.JOB_LOGZ64, seqs, P, masks)
    for c, v in zip(cases, z):
        assert abs(v - c["logz64"]) <= 1e-9 * abs(c["logz64"]), (len(c["seq"]), v, c["logz64"])
    for c, m in zip(cases, masks):
        _, POST = oracle.posterior(c["seq"], P, m)
        assert hashlib.sha256(np.ascontiguousarray(POST, np.float32).tobytes()).hexdigest() == c["post_sha256"]


def test_oracle_matches_reference_long(long_cases, P, oracle):
    _check(long_cases, P, oracle)


def test_oracle_matches_reference_800_and_1000_nt(P, oracle):
    cases = _load("xlong.json")
    assert [len(c["seq"]) for c in cases] == [800, 1000] and cases[1]["mask"] is not None
    _check(cases, P, oracle)
