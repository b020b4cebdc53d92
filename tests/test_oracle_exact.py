"""CPU: the oracle's exact (FP64, exact log1p/exp) pair probabilities, the
reference distribution of the sampler tests, against an independent route --
FP64 central differences of logZ with a per-position unpaired bonus:
P(k unpaired) = d logZ / d u_k = 1 - sum_j P(k, j)."""
import numpy as np


def test_bpp_exact_matches_unpaired_derivative(P, oracle):
    rng = np.random.default_rng(21)
    for L, masked in ((37, False), (80, True)):
        seq = "".join(rng.choice(list("ACGU"), size=L))
        mask = (rng.random(L) < 0.1).astype(np.int8) if masked else None
        M = oracle.bpp_exact(seq, P, mask)
        assert np.all(M >= 0) and np.all(M <= 1) and np.all(np.tril(M) == 0)
        punp = 1.0 - M.sum(0) - M.sum(1)
        h = 1e-5
        for k in range(0, L, 7):
            up = np.zeros(L)
            um = np.zeros(L)
            up[k] = h
            um[k] = -h
            fd = (oracle.logz64_bonus(seq, P, up, mask) - oracle.logz64_bonus(seq, P, um, mask)) / (2 * h)
            assert abs(fd - punp[k]) < 1e-7, (L, k, fd, punp[k])


def test_bpp_exact_close_to_fast_posterior(P, oracle):
    """The reference's float32 posterior approximates the exact one (Fast_Exp /
    Fast_LogPlusEquals): within a few 1e-3 per pair on a 60-nt sequence."""
    rng = np.random.default_rng(22)
    seq = "".join(rng.choice(list("ACGU"), size=60))
    assert np.max(np.abs(oracle.bpp_exact(seq, P) - oracle.bpp(seq, P))) < 5e-3
