"""Pin the oracle (C restatement of gpu_contrafold/cpu.py) to the golden vectors
produced by the reference itself (tests/golden/make_golden.py).  CPU only."""
import hashlib

import numpy as np
import pytest

from conftest import golden_post, mask_of


def test_param_blob_matches_reference_loader(P, golden):
    """contrafold_gpu_gb300.params.load == gpu_contrafold.cpu.load (cpu.py:40-135), bitwise."""
    from contrafold_gpu_gb300 import params
    blob = params.pack64(P)
    assert hashlib.sha256(blob.tobytes()).hexdigest() == golden["params_blob64_sha256"]
    import os
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "params_blob64.npy"))
    assert np.array_equal(ref.view(np.uint64), blob.view(np.uint64))
    assert params.BLOB_LEN == 2577


def test_known_answers(P, oracle):
    # README.md:101,104 of the reference; logZ of cpu.py on this sequence 3.056610
    assert oracle.mfe("GGGGAAAACCCC", P) == "((((....))))"
    assert oracle.mea("GGGGAAAACCCC", P) == "((((....))))"
    assert abs(oracle.logz64("GGGGAAAACCCC", P) - 3.05661) < 1e-5


def test_oracle_logz64_golden(P, golden, oracle):
    for rec in golden["cases"]:
        z = oracle.logz64(rec["seq"], P, mask_of(rec))
        assert abs(z - rec["logz64"]) <= 1e-9 * max(1.0, abs(rec["logz64"])), rec["seq"]


def test_oracle_mfe_golden(P, golden, oracle):
    bad = [r["seq"] for r in golden["cases"] if oracle.mfe(r["seq"], P, mask_of(r)) != r["mfe"]]
    assert not bad, bad[:3]


def test_oracle_posterior_bitwise_golden(P, golden, oracle):
    """FP32 posterior matrix bitwise equal to cpu.posterior (cpu.py:583-820)."""
    for rec in golden["cases"]:
        _, POST = oracle.posterior(rec["seq"], P, mask_of(rec))
        assert hashlib.sha256(np.ascontiguousarray(POST).tobytes()).hexdigest() == rec["post_sha256"], rec["seq"]
        if "post_b64" in rec:
            assert np.array_equal(POST.view(np.uint32), golden_post(rec).view(np.uint32))


def test_oracle_mea_golden(P, golden, oracle):
    """MEA structures bit-exact with cpu.mea at every recorded gamma."""
    n = 0
    for rec in golden["cases"]:
        for g, want in rec["mea"].items():
            assert oracle.mea(rec["seq"], P, float(g), mask_of(rec)) == want, (rec["seq"], g)
            n += 1
    assert n > 250


def test_golden_covers_edge_cases(golden):
    seqs = [r["seq"] for r in golden["cases"]]
    assert "" in seqs and "A" in seqs
    assert any("N" in s for s in seqs)
    assert any(r["mask"] is not None for r in golden["cases"])
    assert max(len(s) for s in seqs) >= 200
    assert len(golden["cases"]) >= 200


def test_oracle_batch_driver(P, golden, oracle):
    """The threaded batch runner (CPU baseline) returns what the single calls return."""
    recs = golden["cases"][20:60]
    seqs = [r["seq"] for r in recs]
    masks = [mask_of(r) for r in recs]
    mea = oracle.batch(oracle.JOB_MEA, seqs, P, masks, 6.0, threads=4)
    assert mea == [r["mea"]["6.0"] for r in recs]
    mfe = oracle.batch(oracle.JOB_MFE, seqs, P, masks, threads=3)
    assert mfe == [r["mfe"] for r in recs]
    z = oracle.batch(oracle.JOB_LOGZ64, seqs, P, masks, threads=2)
    assert np.allclose(z, [r["logz64"] for r in recs], atol=1e-9, rtol=0)


@pytest.mark.parametrize("x", [0.0, 1e-8, 0.3, 0.6615367791, 1.0, 1.6320158198, 2.0, 3.3792499610, 5.0,
                               7.8162726752, 11.0, 11.8624794162, 12.0, 50.0])
def test_lse32_segment_boundaries(oracle, x):
    """Fast_LogPlusEquals: close to log(e^a + e^b) inside the table, exact cut-off beyond it."""
    a, b = np.float32(x), np.float32(0.0)
    r = oracle.lib().oracle_lse32(float(a), float(b))
    exact = np.logaddexp(np.float64(a), 0.0)
    if x >= 11.8624794162:
        assert r == np.float32(a)
    else:
        assert abs(r - exact) < 2e-4
