"""GPU parity: the CUDA engine (through the C-ABI) against the golden vectors of
the reference and against the oracle on seeded batches.

Tolerances (stated by the fold contract):
  logZ FP32 (cf_logz) vs the FP64 engine  <= 5e-4 absolute
  logZ of the posterior     bitwise equal to the oracle's float32 inside (Fast_LogPlusEquals)
  logZ FP64                 <= 1e-9 relative (CUDA vs glibc log1p/exp)
  BPP                       bitwise equal to the reference float32 posterior (=> max-abs 0 <= 1e-4)
  MEA / Viterbi             dot-brackets identical
"""
import hashlib

import numpy as np
import pytest

from conftest import golden_post, mask_of

pytestmark = pytest.mark.gpu


PATHS = ["plain", "warp", "cta", "group", "cluster"]


def set_path(engine, path):
    """plain = per-phase kernels, one sequence per CTA; warp / cta =
    the persistent batched kernels; group / cluster = the grouped kernels on
    one CTA / on a thread-block cluster."""
    if path == "plain":
        engine.set_mode("plain")
    else:
        engine.set_mode("batched")
        engine.set_schedule(path)


@pytest.fixture(autouse=True)
def _reset_engine(request):
    yield
    if "engine" in request.fixturenames:
        eng = request.getfixturevalue("engine")
        eng.set_mode("batched")
        eng.set_schedule("auto")
        eng.set_budget(0)


def _batch(recs):
    from contrafold_gpu_gb300.engine import Batch
    return Batch([r["seq"] for r in recs], [mask_of(r) for r in recs])


def _rand_batch(seed, n, lo, hi, p_mask=0.0, alphabet="ACGU"):
    rng = np.random.default_rng(seed)
    seqs, masks = [], []
    al = np.array(list(alphabet))
    for _ in range(n):
        L = int(rng.integers(lo, hi + 1))
        seqs.append("".join(rng.choice(al, size=L)))
        masks.append((rng.random(L) < p_mask).astype(np.int8) if p_mask > 0 else None)
    return seqs, masks


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_golden_logz64(engine, golden, mode):
    engine.set_mode(mode)
    recs = golden["cases"]
    z = engine.logz64(_batch(recs))
    for r, v in zip(recs, z):
        assert abs(v - r["logz64"]) <= 1e-9 * max(1.0, abs(r["logz64"])), r["seq"]


@pytest.mark.parametrize("path", PATHS)
def test_golden_logz32_tolerance(engine, golden, path):
    set_path(engine, path)
    recs = golden["cases"]
    z = engine.logz(_batch(recs))
    for r, v in zip(recs, z):
        err = abs(float(v) - r["logz64"])
        assert err <= 5e-4, (r["seq"], err)


@pytest.mark.parametrize("path", PATHS)
def test_golden_bpp_bitwise(engine, golden, path):
    set_path(engine, path)
    recs = golden["cases"]
    mats, _ = engine.bpp(_batch(recs))
    for r, M in zip(recs, mats):
        L = len(r["seq"])
        full = np.zeros((L + 2, L + 2), np.float32)
        full[1:L + 1, 1:L + 1] = M
        assert hashlib.sha256(full.tobytes()).hexdigest() == r["post_sha256"], r["seq"]
        if "post_b64" in r:
            ref = golden_post(r)[1:L + 1, 1:L + 1]
            assert np.array_equal(ref.view(np.uint32), M.view(np.uint32))


@pytest.mark.parametrize("path", PATHS)
def test_golden_mea(engine, golden, path):
    set_path(engine, path)
    recs = golden["cases"]
    gammas = sorted({g for r in recs for g in r["mea"]}, key=float)
    for g in gammas:
        sub = [r for r in recs if g in r["mea"]]
        got = engine.mea(_batch(sub), float(g))
        bad = [r["seq"] for r, s in zip(sub, got) if s != r["mea"][g]]
        assert not bad, (g, bad[:3])


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_golden_mfe(engine, golden, mode):
    engine.set_mode(mode)
    recs = golden["cases"]
    got = engine.mfe(_batch(recs))
    bad = [r["seq"] for r, s in zip(recs, got) if s != r["mfe"]]
    assert not bad, bad[:3]


def test_random_batch_vs_oracle(engine, P, oracle):
    """200 seeded sequences (20-150 nt, 10% mask): posterior logZ bitwise vs the
    oracle's float32 inside, cf_logz within 5e-4 of FP64, BPP bitwise, MEA and
    Viterbi identical."""
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = _rand_batch(11, 200, 20, 150, 0.1)
    B = Batch(seqs, masks)
    engine.set_mode("batched")
    z = engine.logz(B)
    mats, z2 = engine.bpp(B)
    mea = engine.mea(B, 6.0)
    mfe = engine.mfe(B)
    zo = oracle.batch(oracle.JOB_LOGZ32, seqs, P, masks)        # Fast_LogPlusEquals, bitwise
    assert np.array_equal(np.float32(zo), z2)
    z64 = oracle.batch(oracle.JOB_LOGZ64, seqs, P, masks)
    assert np.max(np.abs(np.asarray(z, np.float64) - z64)) <= 5e-4
    assert mea == oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0)
    assert mfe == oracle.batch(oracle.JOB_MFE, seqs, P, masks)
    for k in range(0, 200, 37):
        L = len(seqs[k])
        _, POST = oracle.posterior(seqs[k], P, masks[k])
        assert np.array_equal(POST[1:L + 1, 1:L + 1].view(np.uint32), mats[k].view(np.uint32))


def test_plain_equals_batched(engine):
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = _rand_batch(5, 97, 1, 260, 0.1)
    B = Batch(seqs, masks)
    res = {}
    for path in PATHS:
        set_path(engine, path)
        mats, z = engine.bpp(B)
        res[path] = (engine.logz(B), engine.mea(B, 6.0), engine.mfe(B), z, np.concatenate([m.ravel() for m in mats]))
    set_path(engine, "cta")
    engine.set_schedule("auto")
    for path in ("warp", "cta", "group", "cluster"):
        assert np.array_equal(res["plain"][0], res[path][0])
        assert res["plain"][1] == res[path][1]
        assert res["plain"][2] == res[path][2]
        assert np.array_equal(res["plain"][3], res[path][3])
        assert np.array_equal(res["plain"][4].view(np.uint32), res[path][4].view(np.uint32))


def test_edge_cases(engine, P, oracle):
    from contrafold_gpu_gb300.engine import Batch
    seqs = ["", "A", "GC", "NNNN", "GGGGAAAACCCC", "acgu" * 10, "GGGG" + "N" * 30 + "CCCC"]
    B = Batch(seqs)
    z = engine.logz64(B)
    for s, v in zip(seqs, z):
        assert abs(v - oracle.logz64(s, P)) <= 1e-9 * max(1.0, abs(v))
    assert engine.mea(B, 6.0) == [oracle.mea(s, P) for s in seqs]
    assert engine.mfe(B) == [oracle.mfe(s, P) for s in seqs]
    # a fully forced sequence folds to all-unpaired with logZ = L * eu
    Bf = Batch(["GGGGAAAACCCC"], [[1] * 12])
    assert engine.mea(Bf, 6.0) == ["." * 12]
    assert abs(engine.logz64(Bf)[0] - 12 * P["eu"]) < 1e-12


def test_long_sequence_budget_slicing(engine, P, oracle):
    """A small arena budget forces several slices; results are unchanged."""
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = _rand_batch(7, 24, 100, 300, 0.1)
    B = Batch(seqs, masks)
    engine.set_mode("batched")
    full = engine.mea(B, 6.0)
    engine.set_budget(8 << 20)
    try:
        sliced = engine.mea(B, 6.0)
    finally:
        engine.set_budget(0)
    assert full == sliced
    assert full == oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0)


def test_mixed_lengths_every_schedule(engine):
    """A batch mixing 20-250 nt with 257-420 nt sequences gives identical results
    on every schedule (the warp kernel then folds long sequences too)."""
    from contrafold_gpu_gb300.engine import Batch
    s1, m1 = _rand_batch(41, 40, 20, 250, 0.1)
    s2, m2 = _rand_batch(42, 12, 257, 420, 0.1)
    order = np.random.default_rng(43).permutation(len(s1) + len(s2))
    seqs = [(s1 + s2)[k] for k in order]
    masks = [(m1 + m2)[k] for k in order]
    B = Batch(seqs, masks)
    res = {}
    for path in ("auto",) + tuple(PATHS):
        set_path(engine, path)
        mats, zb = engine.bpp(B)
        res[path] = (engine.logz(B).tobytes(), engine.logz64(B).tobytes(), engine.mea(B, 6.0), engine.mfe(B),
                     zb.tobytes(), hashlib.sha256(np.concatenate([m.ravel() for m in mats]).tobytes()).hexdigest(),
                     engine.sample(B, 4, seeds=list(range(len(seqs)))))
    for path in PATHS:
        assert res[path] == res["auto"], path


def test_long_sequence_vs_oracle(engine, P, oracle):
    """One 600-nt sequence (10 % mask): 512-thread per-phase kernels with several
    cells per thread on each diagonal; Viterbi and MEA identical, BPP bitwise,
    FP64 logZ to 1e-9 relative."""
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = _rand_batch(61, 1, 600, 600, 0.1)
    B = Batch(seqs, masks)
    assert engine.mfe(B)[0] == oracle.mfe(seqs[0], P, masks[0])
    assert engine.mea(B, 6.0)[0] == oracle.mea(seqs[0], P, 6.0, masks[0])
    z64 = oracle.logz64(seqs[0], P, masks[0])
    assert abs(engine.logz64(B)[0] - z64) <= 1e-9 * abs(z64)
    # float32 logZ: the 5e-4 of the 200-nt contract, scaled with the length (600 / 200)
    assert abs(engine.logz(B)[0] - z64) <= 5e-4 * 3


def test_long_sequence_cluster_vs_oracle(engine, P, oracle):
    """The cluster schedule (one 8-CTA cluster per sequence) on 600 and 1,000 nt:
    MEA identical to the oracle, BPP bitwise equal to the grouped kernels."""
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = _rand_batch(62, 2, 600, 1000, 0.1)
    B = Batch(seqs, masks)
    try:
        engine.set_schedule("group")
        mats_g, z_g = engine.bpp(B)
        lz_g = engine.logz(B)
        engine.set_schedule("cluster")
        got = engine.mea(B, 6.0)
        mats_c, z_c = engine.bpp(B)
        assert np.array_equal(engine.logz(B), lz_g)
    finally:
        engine.set_schedule("auto")
    assert got[0] == oracle.mea(seqs[0], P, 6.0, masks[0])
    assert z_c.tobytes() == z_g.tobytes()
    for a, b in zip(mats_c, mats_g):
        assert a.tobytes() == b.tobytes()


def test_queue_schedule_refused(engine, tmp_path):
    """The queue schedule is disabled: the engine refuses it (no launch), and a
    schedule table naming it is rejected."""
    from contrafold_gpu_gb300.engine import EngineError
    with pytest.raises(EngineError):
        engine.set_schedule("queue")
    t = tmp_path / "q.txt"
    t.write_text("0 400 1 0 any all queue 0 0\n")
    with pytest.raises(EngineError):
        engine.load_tuning(str(t))


def test_bpp_batch_float64(engine, P):
    """gpu.bpp_batch returns float64 (L, L) matrices (the reference's bpp
    dtype, cpu.py:929), each the device's float32 matrix widened exactly."""
    from contrafold_gpu_gb300 import gpu
    from contrafold_gpu_gb300.engine import Batch
    seqs, masks = _rand_batch(81, 40, 1, 120, 0.1)
    got = gpu.bpp_batch(seqs, P, masks)
    want, _ = engine.bpp(Batch(seqs, masks))
    assert len(got) == len(seqs)
    for g, w, s in zip(got, want, seqs):
        assert g.dtype == np.float64 and g.shape == (len(s), len(s))
        assert np.array_equal(g, w.astype(np.float64))
