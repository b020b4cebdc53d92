"""Sampler checks: structure validity, forced-unpaired masks, reproducibility and
pair frequencies against the exact pair probabilities within 3 sigma binomial
noise (the reference's own checks 3 and 4, tests/test_validation.py:44-76)."""
import numpy as np
import pytest

from conftest import check_pair_frequencies

pytestmark = pytest.mark.gpu


def _pairs(db):
    st, out = [], []
    for k, ch in enumerate(db):
        if ch == "(":
            st.append(k)
        elif ch == ")":
            out.append((st.pop(), k))
    assert not st
    return out


def test_sample_valid_and_reproducible(engine, P):
    from contrafold_gpu_gb300.engine import Batch
    from contrafold_gpu_gb300.params import CODE
    rng = np.random.default_rng(3)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(L))) for L in (12, 50, 133, 260)]
    B = Batch(seqs)
    a = engine.sample(B, 16, seed=7)
    b = engine.sample(B, 16, seed=7)
    c = engine.sample(B, 16, seed=8)
    assert a == b
    assert a != c
    canon = {(0, 3), (3, 0), (1, 2), (2, 1), (2, 3), (3, 2)}
    for s, ss in zip(seqs, a):
        for db in ss:
            assert len(db) == len(s)
            for x, y in _pairs(db):
                assert (CODE[s[x]], CODE[s[y]]) in canon


def test_sample_plain_equals_batched(engine):
    """The per-sequence kernels and the fused warp kernel draw identical samples
    (same inside tables bit for bit, same Philox streams)."""
    from contrafold_gpu_gb300.engine import Batch
    rng = np.random.default_rng(9)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(L))) for L in (5, 33, 90, 201)]
    masks = [None, (rng.random(33) < 0.2).astype(np.int8), None, None]
    B = Batch(seqs, masks)
    out = {}
    for mode in ("plain", "batched"):
        engine.set_mode(mode)
        out[mode] = engine.sample(B, 8, seed=123)
    engine.set_mode("batched")
    assert out["plain"] == out["batched"]


def test_sample_forced_unpaired_mask(engine, golden):
    """check [4] of the reference validation script: zero violations."""
    from contrafold_gpu_gb300.engine import Batch
    v = golden["validation_script"]
    s4, m4 = v["check4_seq"], v["check4_mask"]
    out = engine.sample(Batch([s4], [m4]), 2000, seed=2)[0]
    viol = sum(1 for db in out for k, ch in enumerate(db) if m4[k] and ch != ".")
    assert viol == 0


@pytest.mark.parametrize("seq,n", [("GCGCGCAAAAGCGCGCAAAAGCGC", 20000)])
def test_sample_frequencies_match_posterior(engine, P, oracle, seq, n):
    """Pair frequencies vs the exact pair probabilities (the distribution the
    sampler draws from): per pair within 3 sigma + 1/N (conftest.check_pair_frequencies)."""
    from contrafold_gpu_gb300.engine import Batch
    out = engine.sample(Batch([seq]), n, seed=1)[0]
    check_pair_frequencies(out, oracle.bpp_exact(seq, P), n)


def test_sample_frequencies_random_masked(engine, P, oracle):
    from contrafold_gpu_gb300.engine import Batch
    rng = np.random.default_rng(17)
    L, n = 60, 8000
    seq = "".join(rng.choice(list("ACGU"), size=L))
    mask = (rng.random(L) < 0.1).astype(np.int8)
    out = engine.sample(Batch([seq], [mask]), n, seed=5)[0]
    check_pair_frequencies(out, oracle.bpp_exact(seq, P, mask), n)


def test_sample_warp_schedule_equals_grouped(engine):
    """The warp-persistent kernel (inside and samples in one launch) and the
    grouped inside + k_sample32 draw identical samples: same tables bit for
    bit, same Philox streams."""
    from contrafold_gpu_gb300.engine import Batch
    rng = np.random.default_rng(23)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(L))) for L in rng.integers(1, 300, 40)]
    masks = [(rng.random(len(s)) < 0.1).astype(np.int8) if k % 3 == 0 else None for k, s in enumerate(seqs)]
    B = Batch(seqs, masks)
    out = {}
    try:
        for sched in ("group", "warp"):
            engine.set_schedule(sched)
            out[sched] = (engine.sample(B, 9, seed=31), engine.sample(B, 4, seeds=list(range(500, 540))))
    finally:
        engine.set_schedule("auto")
    assert out["group"] == out["warp"]


def test_fold_tasks_one_submission_equals_chunked(P):
    """fold_tasks_gpu submits every task at once; its samples equal the
    reference's chunked loop (tasks sorted by length, chunk c0 sampled with
    seed + c0) on 10,000 mixed-length tasks, masks on every third."""
    import contrafold_gpu_gb300 as cg
    from contrafold_gpu_gb300 import gpu
    rng = np.random.default_rng(23)
    lens = rng.integers(20, 301, 10000)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(L))) for L in lens]
    masks = [(rng.random(len(s)) < 0.1).astype(np.int8) if k % 3 == 0 else None for k, s in enumerate(seqs)]
    one = cg.fold_tasks_gpu(seqs, masks, P, chunk=4096, seed=5)
    chunked = gpu.fold_tasks_chunked(seqs, masks, P, chunk=4096, seed=5)
    assert one == chunked
    assert all(db[k] == "." for db, m in zip(one, masks) if m is not None for k in np.nonzero(m)[0])


def test_fold_tasks_gpu_api(P):
    import contrafold_gpu_gb300 as cg
    pytest.importorskip("torch")
    seqs = ["GGGGAAAACCCC", "ACGUACGUAC", "GGGGAAAACCCCGGGGAAAACCCC"]
    out = cg.fold_tasks_gpu(seqs, [None, [1] * 10, None], P, chunk=2, seed=3)
    assert [len(s) for s in out] == [len(s) for s in seqs]
    assert out[1] == "." * 10
