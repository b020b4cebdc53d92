"""The schedule table (cf_engine_load_tuning): a written table changes the
schedule the automatic path picks, results stay identical, malformed tables
are rejected and leave the table unchanged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(n, L, seed):
    from contrafold_gpu_gb300.engine import Batch
    rng = np.random.default_rng(seed)
    seqs = ["".join(rng.choice(list("ACGU"), size=L)) for _ in range(n)]
    masks = [(rng.random(L) < 0.1).astype(np.int8) for _ in range(n)]
    return Batch(seqs, masks)


def _schedule(eng, job, B):
    from contrafold_gpu_gb300.engine import Plan
    p = Plan(eng, job, B.offsets)
    try:
        return p.schedule
    finally:
        p.close()


def test_written_table_changes_schedule(P, tmp_path):
    from contrafold_gpu_gb300.engine import CF_JOB_LOGZ, CF_JOB_MEA, Engine
    eng = Engine(P)
    B = _batch(64, 120, 3)
    assert eng.tuning_rows == 5
    assert _schedule(eng, CF_JOB_MEA, B) == "group"          # built-in: uniform batches fold grouped
    want_mea, want_z = eng.mea(B, 6.0), eng.logz(B)
    t = tmp_path / "tuning.txt"
    t.write_text("# test table\n"
                 "0 150 32 0 uniform mea warp 0 0   # uniform MEA batches of >= 32 up to 150 nt: warp kernel\n"
                 "0 150 1 0 any logz cta 0 2\n")
    eng.load_tuning(str(t))
    assert eng.tuning_rows == 2
    assert _schedule(eng, CF_JOB_MEA, B) == "warp"
    assert _schedule(eng, CF_JOB_LOGZ, B) == "cta"
    assert eng.mea(B, 6.0) == want_mea
    assert np.array_equal(eng.logz(B), want_z)
    # an explicit schedule still overrides the table
    eng.set_schedule("group")
    assert _schedule(eng, CF_JOB_MEA, B) == "group"
    eng.set_schedule("auto")
    eng.load_tuning(None)
    assert eng.tuning_rows == 5 and _schedule(eng, CF_JOB_MEA, B) == "group"
    eng.close()


@pytest.mark.parametrize("text", ["0 150 32 0 uniform mea warp 0\n",            # 8 fields
                                  "0 150 32 0 sometimes mea warp 0 0\n",        # bad uniform
                                  "0 150 32 0 any mea,viterbi warp 0 0\n",      # bad job
                                  "0 150 32 0 any mea fast 0 0\n",              # bad schedule
                                  "0 150 x 0 any mea warp 0 0\n",               # bad number
                                  "0 150 32 0 any mea group 99 0\n"])           # group above 32
def test_malformed_table_rejected(P, tmp_path, text):
    from contrafold_gpu_gb300.engine import Engine, EngineError
    eng = Engine(P)
    t = tmp_path / "bad.txt"
    t.write_text(text)
    with pytest.raises(EngineError):
        eng.load_tuning(str(t))
    assert eng.tuning_rows == 5
    with pytest.raises(EngineError):
        eng.load_tuning(str(tmp_path / "missing.txt"))
    eng.close()


def test_table_from_environment(P, tmp_path, monkeypatch):
    from contrafold_gpu_gb300.engine import CF_JOB_MEA, Engine
    t = tmp_path / "env.txt"
    t.write_text("0 150 1 0 any all warp 0 0\n")
    monkeypatch.setenv("CONTRAFOLD_GB300_TUNING", str(t))
    eng = Engine(P)
    assert eng.tuning_rows == 1
    assert _schedule(eng, CF_JOB_MEA, _batch(8, 100, 4)) == "warp"
    eng.close()
