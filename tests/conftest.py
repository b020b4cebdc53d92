import base64
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden", "golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def P():
    from contrafold_gpu_gb300 import params
    return params.load()


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


def golden_post(rec):
    """The reference's float32 POST matrix ((L+2) x (L+2)) stored in a golden record."""
    L = len(rec["seq"])
    raw = base64.b64decode(rec["post_b64"])
    return np.frombuffer(raw, np.float32).reshape(L + 2, L + 2)


def mask_of(rec):
    m = rec.get("mask")
    return None if m is None else [int(c) for c in m]


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def engine(P):
    if not _gpu_available():
        pytest.skip("no CUDA device")
    from contrafold_gpu_gb300 import build, engine as E
    build.build()
    return E.Engine(P)
