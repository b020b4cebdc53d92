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


def pairs_of(db):
    """(i, j) 0-based pairs of a dot-bracket."""
    st, out = [], []
    for k, ch in enumerate(db):
        if ch == "(":
            st.append(k)
        elif ch == ")":
            out.append((st.pop(), k))
    assert not st
    return out


def binom_quantile(K, q, tail):
    """Smallest c with P(Binomial(K, q) > c) <= tail."""
    import math
    logp = [math.lgamma(K + 1) - math.lgamma(c + 1) - math.lgamma(K - c + 1) + c * math.log(q)
            + (K - c) * math.log1p(-q) for c in range(K + 1)]
    above = 0.0
    for c in range(K, -1, -1):       # P(X > c - 1) accumulated from the top
        above += math.exp(logp[c])
        if above > tail:
            return c
    return 0


def check_pair_frequencies(samples, p, n):
    """Per pair: |f - p| <= 3 sqrt(p (1 - p) / N) + 1/N.  Pairs are many (up to
    L^2 / 2), and a 3-sigma band holds for ~99.7 % of them by construction, so
    the test allows as many exceedances as a Binomial(K, 0.003) stays under
    with probability 1 - 1e-6 (K = pairs with p >= 1/N, the only ones that can
    leave the band), and none beyond 5 sigma + 1/N."""
    L = p.shape[0]
    f = np.zeros((L, L))
    for db in samples:
        for x, y in pairs_of(db):
            f[x, y] += 1
    f /= n
    sig = np.sqrt(p * (1 - p) / n)
    out3 = np.abs(f - p) > 3 * sig + 1.0 / n
    out5 = np.abs(f - p) > 5 * sig + 1.0 / n
    K = int(np.count_nonzero(p >= 1.0 / n))
    allowed = binom_quantile(K, 0.003, 1e-6)
    assert int(out5.sum()) == 0, np.argwhere(out5)[:5]
    assert int(out3.sum()) <= allowed, (int(out3.sum()), allowed, K)
    return int(out3.sum()), K
