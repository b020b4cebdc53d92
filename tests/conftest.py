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


def binom_upper_tail(N, p, c):
    """P(Binomial(N, p) >= c), summed from the pmf (c small)."""
    import math
    if c <= 0:
        return 1.0
    if p <= 0.0:
        return 0.0
    lp, lq = math.log(p), math.log1p(-p)
    tot, x = 0.0, c
    while x <= N:
        t = math.exp(math.lgamma(N + 1) - math.lgamma(x + 1) - math.lgamma(N - x + 1) + x * lp + (N - x) * lq)
        tot += t
        if x > c + 10 and t < 1e-18 * max(tot, 1e-300):
            break
        x += 1
    return min(1.0, tot)


def check_pair_frequencies(samples, p, n):
    """Sampled pair frequencies f against pair probabilities p, N = n samples.

    Pairs with N p >= 10 (where the binomial count is close to normal): per
    pair |f - p| <= 3 sqrt(p (1 - p) / N) + 1/N.  A 3-sigma band holds for
    ~99.7 % of pairs by construction, so as many exceedances are allowed as a
    Binomial(K, 0.003) stays under with probability 1 - 1e-6 (K = such pairs),
    and none beyond 5 sigma + 1/N.
    Pairs with N p < 10 (Poisson regime: the normal band would understate the
    upper tail): the observed count c must have an upper-tail probability
    P(Binomial(N, p) >= c) >= 1e-6 / K_small (Bonferroni over the K_small such
    pairs seen), and a pair of probability 0 is never drawn.
    Returns (3-sigma exceedances, K)."""
    L = p.shape[0]
    cnt = np.zeros((L, L))
    for db in samples:
        for x, y in pairs_of(db):
            cnt[x, y] += 1
    f = cnt / n
    normal = n * p >= 10
    sig = np.sqrt(p * (1 - p) / n)
    out3 = normal & (np.abs(f - p) > 3 * sig + 1.0 / n)
    out5 = normal & (np.abs(f - p) > 5 * sig + 1.0 / n)
    K = int(np.count_nonzero(normal))
    allowed = binom_quantile(K, 0.003, 1e-6)
    assert int(out5.sum()) == 0, [(int(a), int(b), float(f[a, b]), float(p[a, b])) for a, b in np.argwhere(out5)[:5]]
    assert int(out3.sum()) <= allowed, (int(out3.sum()), allowed, K)
    impossible = (p == 0) & (cnt > 0)
    assert not impossible.any(), np.argwhere(impossible)[:5]
    small = np.argwhere(~normal & (cnt > 0) & (p > 0))
    thr = 1e-6 / max(1, len(small))
    for a, b in small:
        tail = binom_upper_tail(n, float(p[a, b]), int(cnt[a, b]))
        assert tail >= thr, (int(a), int(b), int(cnt[a, b]), float(p[a, b]), tail)
    return int(out3.sum()), K
