"""Differentiation: tying Jacobian (CPU) and GPU gradients against FP64 central
finite differences of the oracle (h = 1e-4) and the posterior identities
d logZ / d bonus_k = P(k unpaired), d logZ / d bp_XY = sum of P(pairs XY or YX)."""
import numpy as np
import pytest

from contrafold_gpu_gb300 import grad, params


def test_tying_jacobian_is_exact():
    names = grad.feature_names()
    assert len(names) == 708
    J = grad.tying_jacobian(names)
    theta = grad.raw_vector()
    blob = params.pack64(grad.tables_from_vector(theta, names))
    assert np.allclose(J @ theta, blob, atol=1e-12, rtol=0)
    # base_pair_AU feeds bp[A][U] and bp[U][A]
    f = names.index("base_pair_AU")
    nz = np.nonzero(J[:, f])[0]
    assert sorted(nz.tolist()) == sorted([params.OFFSETS["bp"] + 0 * 5 + 3, params.OFFSETS["bp"] + 3 * 5 + 0])


def test_write_params_roundtrip(tmp_path):
    names = grad.feature_names()
    theta = grad.raw_vector() * 1.5
    p = tmp_path / "p.params"
    grad.write_params(str(p), theta, names)
    assert np.allclose(grad.raw_vector(str(p)), theta, rtol=1e-9)


def _fd_theta(oracle, P, seq, bonus, names, theta, f, h=1e-4):
    tp = theta.copy(); tp[f] += h
    tm = theta.copy(); tm[f] -= h
    bp = params.pack64(grad.tables_from_vector(tp, names))
    bm = params.pack64(grad.tables_from_vector(tm, names))
    return (oracle.logz64_bonus(seq, P, bonus, blob64=bp) - oracle.logz64_bonus(seq, P, bonus, blob64=bm)) / (2 * h)


@pytest.mark.gpu
def test_grad_vs_fp64_finite_differences(engine, P, oracle):
    rng = np.random.default_rng(3)
    names = grad.feature_names()
    theta = grad.raw_vector()
    seqs = ["".join(rng.choice(list("ACGU"), size=L)) for L in (60, 110)]
    bonus = [rng.normal(0, 0.5, size=len(s)).astype(np.float32) for s in seqs]
    res = grad.logz_grad(seqs, theta, bonus)
    # logZ with bonus vs the FP64 oracle
    for b, s in enumerate(seqs):
        z64 = oracle.logz64_bonus(s, P, bonus[b].astype(np.float64))
        assert abs(res.logz[b] - z64) < 5e-4
    # bonus gradient: central differences on a few positions
    h = 1e-4
    for b, s in enumerate(seqs):
        u = bonus[b].astype(np.float64)
        for k in (0, len(s) // 3, len(s) - 1):
            up, um = u.copy(), u.copy()
            up[k] += h
            um[k] -= h
            fd = (oracle.logz64_bonus(s, P, up) - oracle.logz64_bonus(s, P, um)) / (2 * h)
            assert abs(res.d_bonus[b][k] - fd) < 2e-3, (b, k, res.d_bonus[b][k], fd)
    # raw-feature gradient: the features every structure touches plus a seeded sample
    pick = [names.index(k) for k in ("multi_base", "multi_unpaired", "multi_paired", "external_unpaired",
                                     "external_paired", "base_pair_GU", "base_pair_CG", "hairpin_length_at_least_3")]
    pick += list(np.random.default_rng(7).choice(len(names), 10, replace=False))
    b = 0
    for f in pick:
        fd = _fd_theta(oracle, P, seqs[b], bonus[b].astype(np.float64), names, theta, f)
        assert abs(res.d_theta[b, f] - fd) < 2e-3 + 2e-3 * abs(fd), (names[f], res.d_theta[b, f], fd)


@pytest.mark.gpu
def test_grad_posterior_identities(engine, P, oracle):
    """Without bonuses, d logZ / d bp_XY is the expected number of XY pairs and
    d logZ / d u_k is P(k unpaired).  Against the FP64 oracle (finite
    differences) the counts must match tightly.  The reference's own posterior
    (Fast_Exp / Fast_LogPlusEquals arithmetic) is biased against the exact
    expectation -- measured 1-6 % on these sums, e.g. GU pairs of the 90-nt
    sequence: exact 0.59782, Fast posterior 0.56393 -- so the posterior-derived
    counts are checked within 10 %."""
    from contrafold_gpu_gb300.engine import Batch
    rng = np.random.default_rng(5)
    seqs = ["".join(rng.choice(list("ACGU"), size=L)) for L in (40, 90, 150)]
    masks = [None, (rng.random(90) < 0.1).astype(np.int8), None]
    res = grad.logz_grad(seqs, None, None, masks)
    mats, _ = engine.bpp(Batch(seqs, masks))
    names = grad.feature_names()
    theta = grad.raw_vector()
    feat = {(0, 3): "base_pair_AU", (1, 2): "base_pair_CG", (2, 3): "base_pair_GU"}
    o = params.OFFSETS["bp"]
    for b, s in enumerate(seqs):
        M = mats[b].astype(np.float64)
        punp = 1.0 - M.sum(0) - M.sum(1)
        assert np.max(np.abs(res.d_bonus[b] - punp)) < 1.5e-2
        # every position is paired or unpaired: sum_k P(unpaired) = L - 2 E[#pairs] (float32 tables)
        assert abs(res.d_bonus[b].sum() - (len(s) - 2 * sum(res.d_blob[b, o:o + 25]))) < 1e-4 * len(s)
        code = [params.CODE.get(c, 4) for c in s]
        for (x, y), fname in feat.items():
            got = res.d_blob[b, o + x * 5 + y] + res.d_blob[b, o + y * 5 + x]
            f = names.index(fname)
            h = 1e-5
            tp, tm = theta.copy(), theta.copy()
            tp[f] += h
            tm[f] -= h
            exact = (oracle.logz64_bonus(s, P, None, masks[b], blob64=params.pack64(grad.tables_from_vector(tp, names)))
                     - oracle.logz64_bonus(s, P, None, masks[b], blob64=params.pack64(grad.tables_from_vector(tm, names)))) / (2 * h)
            assert abs(got - exact) < 1e-3 * max(1.0, exact), (b, fname, got, exact)
            fast = sum(M[i, j] for i in range(len(s)) for j in range(i + 1, len(s)) if {code[i], code[j]} == {x, y})
            assert abs(got - fast) < 5e-3 + 0.1 * fast, (b, fname, got, fast)


@pytest.mark.gpu
def test_autograd_function(engine, P):
    torch = pytest.importorskip("torch")
    LogZ = grad.LogZ
    seqs = ["GGGGAAAACCCCAUGCAUGC", "ACGUACGUAGCUAGCUAGCAUCGAUCG"]
    theta = torch.tensor(grad.raw_vector(), dtype=torch.float64, requires_grad=True)
    bonus = torch.zeros((2, 27), dtype=torch.float32, requires_grad=True)
    z = LogZ.apply(theta, bonus, seqs)
    z.sum().backward()
    res = grad.logz_grad(seqs, None, [np.zeros(20), np.zeros(27)])
    assert np.allclose(theta.grad.numpy(), res.d_theta.sum(0))
    assert np.allclose(bonus.grad[0, :20].numpy(), res.d_bonus[0], atol=1e-6)
    assert float(bonus.grad[0, 20:].abs().sum()) == 0.0


@pytest.mark.gpu
def test_grad_checkpointing_bitwise_and_memory(engine, P):
    """cf_grad on 1,000-nt sequences: FM2 kept on every diagonal, on every 8th
    and on every 32nd gives bitwise the same logZ, counts and unpaired
    probabilities (the counts are exact fixed-point sums, and recomputed FM2
    cells equal the stored ones bit for bit); two runs are identical; the
    checkpointed arena is smaller."""
    from contrafold_gpu_gb300.engine import Engine, grad_arena_bytes
    rng = np.random.default_rng(41)
    seqs = ["".join(rng.choice(list("ACGU"), size=1000)) for _ in range(2)]
    bonus = [rng.normal(0, 0.5, size=1000).astype(np.float32) for _ in seqs]
    masks = [None, (rng.random(1000) < 0.1).astype(np.int8)]
    eng = Engine(P)
    res = {}
    try:
        for every in (1, 8, 32, 8):
            eng.set_grad_checkpoint(every)
            r = grad.logz_grad(seqs, None, bonus, masks, engine=eng)
            res.setdefault(every, []).append((r.logz.tobytes(), r.d_blob.tobytes(),
                                              b"".join(u.tobytes() for u in r.d_bonus)))
    finally:
        eng.close()
    ref = res[1][0]
    assert res[8][0] == ref and res[32][0] == ref
    assert res[8][1] == res[8][0]
    full, ck8 = grad_arena_bytes(1000, 1), grad_arena_bytes(1000, 8)
    tri = 4 * 1001 * 1002 // 2
    assert ck8 < full and ck8 < 5 * tri, (full, ck8, tri)
