"""GPU parity on the measured workloads themselves (contrafold_gpu_gb300.workloads),
through the C-ABI, against the oracle.

  mea_200  (10,000 x 200 nt, Bernoulli(0.1) mask):
           MEA (gamma 6) and Viterbi dot-brackets identical to the oracle on all
           10,000 sequences; BPP bitwise (SHA-256 of the float32 matrix) on 512;
           cf_logz within 5e-4 (absolute) of the FP64 logZ on 1,000.
  sampling (lengths U{40..400}): pair frequencies of sequences of 40, 200 and
           400 nt, with and without a Bernoulli(0.1) mask, against the exact
           Boltzmann pair probabilities, per pair within 3 sigma binomial noise
           plus 1/N (see conftest.check_pair_frequencies for the count of exceedances allowed).
  grad_300 (512 x 300 nt, bonuses N(0, 0.5)): d logZ / d bonus and d logZ /
           d raw feature against FP64 central differences of the oracle
           (h = 1e-4), |err| <= 2e-3 + 2e-3 |fd|; logZ within 5e-4 * 300/200.
"""
import concurrent.futures as cfut
import hashlib
import os

import numpy as np
import pytest

from conftest import check_pair_frequencies, pairs_of
from contrafold_gpu_gb300 import workloads

pytestmark = pytest.mark.gpu

CORES = os.cpu_count() or 1


@pytest.fixture(scope="module")
def mea_workload():
    sb, mask = workloads.mea_200()
    return workloads.as_strings(sb), list(mask)


def test_mea_200_all_structures(engine, P, oracle, mea_workload):
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = mea_workload
    engine.set_mode("batched")
    engine.set_schedule("auto")
    got = engine.mea(Batch(seqs, masks), 6.0)
    want = oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0, threads=CORES)
    bad = [k for k, (a, b) in enumerate(zip(got, want)) if a != b]
    assert not bad, (len(bad), bad[:5])


def test_mea_200_all_viterbi(engine, P, oracle, mea_workload):
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = mea_workload
    engine.set_mode("batched")
    got = engine.mfe(Batch(seqs, masks))
    want = oracle.batch(oracle.JOB_MFE, seqs, P, masks, threads=CORES)
    bad = [k for k, (a, b) in enumerate(zip(got, want)) if a != b]
    assert not bad, (len(bad), bad[:5])


def test_mea_200_bpp_bitwise(engine, P, oracle, mea_workload):
    """The first 512 sequences: every float32 posterior bit equal (SHA-256 per
    matrix), so the max-abs difference is 0 <= 1e-4."""
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = mea_workload
    m = 512
    mats, z = engine.bpp(Batch(seqs[:m], masks[:m]))

    def ref(k):
        zo, POST = oracle.posterior(seqs[k], P, masks[k])
        L = len(seqs[k])
        return zo, hashlib.sha256(np.ascontiguousarray(POST[1:L + 1, 1:L + 1]).tobytes()).hexdigest()

    with cfut.ThreadPoolExecutor(CORES) as ex:     # the oracle releases the GIL in C
        refs = list(ex.map(ref, range(m)))
    for k in range(m):
        assert hashlib.sha256(np.ascontiguousarray(mats[k]).tobytes()).hexdigest() == refs[k][1], k
        assert np.float32(z[k]) == refs[k][0], k


def test_mea_200_logz(engine, P, oracle, mea_workload):
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = mea_workload
    m = 1000
    z = engine.logz(Batch(seqs[:m], masks[:m])).astype(np.float64)
    z64 = oracle.batch(oracle.JOB_LOGZ64, seqs[:m], P, masks[:m], threads=CORES)
    assert np.max(np.abs(z - z64)) <= 5e-4


# ----------------------------------------------------------------------------- sampling
@pytest.mark.parametrize("L,masked,n", [(40, False, 20000), (40, True, 20000), (200, False, 8000),
                                         (200, True, 8000), (400, False, 4000), (400, True, 4000)])
def test_sampling_frequencies(engine, P, oracle, L, masked, n):
    from contrafold_gpu_gb300.engine import Batch
    # a sequence of the sampling workload's alphabet and composition (GC 0.5), seeded by length
    rng = np.random.default_rng(1000 + L)
    seq = workloads.ALPHA[rng.integers(0, 4, L)].tobytes().decode()
    mask = (rng.random(L) < 0.1).astype(np.int8) if masked else None
    engine.set_mode("batched")
    engine.set_schedule("auto")
    out = engine.sample(Batch([seq], None if mask is None else [mask]), n, seed=L)[0]
    if mask is not None:
        assert all(db[k] == "." for db in out for k in np.nonzero(mask)[0])
    p = oracle.bpp_exact(seq, P, mask)
    check_pair_frequencies(out, p, n)


def test_sampling_workload_sequences(engine, P, oracle):
    """Three sequences of the sampling workload itself (the shortest, the median,
    the longest), 100 samples each as in the benchmark, pooled over 40 seeds."""
    from contrafold_gpu_gb300.engine import Batch
    seqs = workloads.sampling()
    lens = np.array([len(s) for s in seqs])
    pick = [int(np.argmin(lens)), int(np.argsort(lens)[len(lens) // 2]), int(np.argmax(lens))]
    sub = [seqs[k] for k in pick]
    pooled = [[] for _ in sub]
    for seed in range(40):
        res = engine.sample(Batch(sub), 100, seed=seed)
        for k in range(len(sub)):
            pooled[k] += res[k]
    for k, s in enumerate(sub):
        check_pair_frequencies(pooled[k], oracle.bpp_exact(s, P), 4000)


# ----------------------------------------------------------------------------- gradients
def test_grad_300_vs_fp64_finite_differences(engine, P, oracle):
    from contrafold_gpu_gb300 import grad, params
    seqs, bonus = workloads.grad_300()
    pick_seq = [0, 1]
    sub = [seqs[b] for b in pick_seq]
    ub = [bonus[b] for b in pick_seq]
    names = grad.feature_names()
    theta = grad.raw_vector()
    res = grad.logz_grad(sub, theta, ub)
    h = 1e-4
    feats = [names.index(k) for k in ("multi_base", "multi_unpaired", "multi_paired", "external_unpaired",
                                      "external_paired", "base_pair_GU", "base_pair_CG", "hairpin_length_at_least_3")]
    feats += [int(f) for f in np.random.default_rng(8).choice(len(names), 8, replace=False)]

    def fd_bonus(b, k):
        u = ub[b].astype(np.float64)
        up, um = u.copy(), u.copy()
        up[k] += h
        um[k] -= h
        return (oracle.logz64_bonus(sub[b], P, up) - oracle.logz64_bonus(sub[b], P, um)) / (2 * h)

    def fd_theta(b, f):
        tp, tm = theta.copy(), theta.copy()
        tp[f] += h
        tm[f] -= h
        u = ub[b].astype(np.float64)
        zp = oracle.logz64_bonus(sub[b], P, u, blob64=params.pack64(grad.tables_from_vector(tp, names)))
        zm = oracle.logz64_bonus(sub[b], P, u, blob64=params.pack64(grad.tables_from_vector(tm, names)))
        return (zp - zm) / (2 * h)

    L = len(sub[0])
    jobs = [("u", b, k) for b in range(2) for k in (0, L // 4, L // 2, L - 1)] + \
           [("t", b, f) for b in range(2) for f in feats]
    with cfut.ThreadPoolExecutor(CORES) as ex:
        fds = list(ex.map(lambda j: fd_bonus(j[1], j[2]) if j[0] == "u" else fd_theta(j[1], j[2]), jobs))
    for (kind, b, x), fd in zip(jobs, fds):
        got = res.d_bonus[b][x] if kind == "u" else res.d_theta[b, x]
        assert abs(got - fd) <= 2e-3 + 2e-3 * abs(fd), (kind, b, x if kind == "u" else names[x], got, fd)
    for b in range(2):
        z64 = oracle.logz64_bonus(sub[b], P, ub[b].astype(np.float64))
        assert abs(res.logz[b] - z64) <= 5e-4 * 300 / 200
