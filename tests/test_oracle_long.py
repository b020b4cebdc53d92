"""Pin the oracle at 300-600 nt to the reference itself (tests/golden/long.json,
made by tests/golden/make_golden.py --long from gpu_contrafold/cpu.py): FP64 logZ
to 1e-9 relative, Viterbi and MEA structures identical, float32 posterior
matrices bitwise (SHA-256).  The GPU tests compare the engine with the oracle at
these lengths (600 nt, 600-1,000 nt on the cluster schedule).  CPU only."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import mask_of

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "long.json")


@pytest.fixture(scope="module")
def long_cases():
    with open(FIXTURE) as fh:
        return json.load(fh)["cases"]


def test_long_fixture_lengths(long_cases):
    assert sorted(len(c["seq"]) for c in long_cases) == [300, 350, 400, 450, 500, 600, 600]


def test_oracle_matches_reference_long(long_cases, P, oracle):
    seqs = [c["seq"] for c in long_cases]
    masks = [mask_of(c) for c in long_cases]
    assert oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0) == [c["mea"]["6.0"] for c in long_cases]
    assert oracle.batch(oracle.JOB_MFE, seqs, P, masks) == [c["mfe"] for c in long_cases]
    z = oracle.batch(oracle.JOB_LOGZ64, seqs, P, masks)
    for c, v in zip(long_cases, z):
        assert abs(v - c["logz64"]) <= 1e-9 * abs(c["logz64"]), (len(c["seq"]), v, c["logz64"])
    for c, m in zip(long_cases, masks):
        _, POST = oracle.posterior(c["seq"], P, m)
        assert hashlib.sha256(np.ascontiguousarray(POST, np.float32).tobytes()).hexdigest() == c["post_sha256"]
