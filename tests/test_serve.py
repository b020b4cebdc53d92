"""Serving loop: every result equals the same request folded alone, open-loop
replay, cancellation, argument errors; the request-stream generator on CPU."""
import numpy as np
import pytest

from contrafold_gpu_gb300 import serve
from contrafold_gpu_gb300.engine import CF_ECANCELLED, Batch, EngineError


def test_mixed_workload_shape():
    reqs, t = serve.mixed_workload(4000, rate=1000.0, seed=0)
    lens = np.array([len(r.seq) for r in reqs])
    assert lens.min() >= 30 and lens.max() <= 1000
    assert 140 <= np.median(lens) <= 160
    ops = np.array([r.op for r in reqs])
    assert abs((ops == "logz").mean() - 0.4) < 0.03 and abs((ops == "sample").mean() - 0.2) < 0.03
    assert abs(np.mean([r.mask is not None for r in reqs]) - 0.1) < 0.02
    assert np.all(np.diff(t) >= 0) and t[0] == 0.0
    assert abs(len(reqs) / t[-1] - 1000.0) < 100.0
    assert all(set(r.seq) <= set("ACGU") for r in reqs[:50])
    # seeded
    r1, t1 = serve.mixed_workload(50, rate=1000.0, seed=0)
    r2, t2 = serve.mixed_workload(50, rate=1000.0, seed=0)
    assert [r.seq for r in r2] == [r.seq for r in r1] and np.array_equal(t1, t2)
    assert [r.seed for r in r2] == [r.seed for r in r1]


def _alone(engine, r):
    B = Batch([r.seq], None if r.mask is None else [r.mask])
    if r.op == "logz":
        return float(engine.logz(B)[0])
    if r.op == "mea":
        return engine.mea(B, r.gamma)[0]
    return engine.sample(B, r.n_samples, seed=r.seed)[0]


def _same(a, b):
    if isinstance(a, float):
        return abs(a - b) <= 1e-5 * max(1.0, abs(b))   # logZ tolerance: float32 rounding
    return a == b


@pytest.mark.gpu
def test_results_equal_alone_runs(engine, P):
    reqs, _ = serve.mixed_workload(160, rate=1e9, seed=4, max_len=420)
    with serve.Server(P, workers=3) as srv:
        srv.pause(True)                     # queue everything, then fold in mixed batches
        tickets = [srv.submit(r) for r in reqs]
        srv.pause(False)
        got = [srv.result(t) for t in tickets]
        st = srv.stats()
    assert st["done"] == len(reqs) and st["batches"] < len(reqs)
    for r, g in zip(reqs, got):
        assert _same(g, _alone(engine, r)), (r.op, len(r.seq))


@pytest.mark.gpu
def test_replay_open_loop(engine, P):
    reqs, t = serve.mixed_workload(400, rate=4000.0, seed=5)
    with serve.Server(P, workers=4) as srv:
        rep = srv.replay(reqs, t)
    assert np.all(rep.status == 0)
    assert np.all(rep.latency_ms > 0)
    for k in range(0, 400, 23):
        assert _same(rep.results[k], _alone(engine, reqs[k])), (k, reqs[k].op)


@pytest.mark.gpu
def test_cancel_and_errors(P):
    with serve.Server(P, workers=2) as srv:
        srv.pause(True)
        a = srv.submit(serve.Request("mea", "GGGGAAAACCCC"))
        b = srv.submit(serve.Request("logz", "GGGGAAAACCCC"))
        c = srv.submit(serve.Request("sample", "GGGGAAAACCCC", n_samples=3, seed=9))
        srv.cancel(b)
        with pytest.raises(EngineError):
            srv.cancel(b)                    # already cancelled
        srv.pause(False)
        assert srv.result(a) == "((((....))))"
        with pytest.raises(EngineError) as ei:
            srv.result(b)
        assert ei.value.code == CF_ECANCELLED
        assert len(srv.result(c)) == 3
        with pytest.raises(EngineError):
            srv.submit(serve.Request("mea", "ACGU", gamma=0.0))
        with pytest.raises(ValueError):
            srv.submit(serve.Request("fold", "ACGU"))
        assert srv.stats()["cancelled"] == 1


@pytest.mark.gpu
def test_batch_trace(P, tmp_path, monkeypatch):
    """CONTRAFOLD_GB300_SERVER_TRACE: one line per batch -- worker, op, bucket,
    requests, nucleotides, longest sequence, start <= end, status -- covering
    every request."""
    trace = tmp_path / "trace.txt"
    monkeypatch.setenv("CONTRAFOLD_GB300_SERVER_TRACE", str(trace))
    reqs, _ = serve.mixed_workload(120, rate=1e9, seed=6, max_len=300)
    with serve.Server(P, workers=2) as srv:
        srv.pause(True)
        tickets = [srv.submit(r) for r in reqs]
        srv.pause(False)
        for t in tickets:
            srv.result(t)
    rows = [line.split() for line in trace.read_text().splitlines()]
    assert rows and all(len(r) == 9 for r in rows)
    assert sum(int(r[3]) for r in rows) == len(reqs)
    assert sum(int(r[4]) for r in rows) == sum(len(r.seq) for r in reqs)
    for r in rows:
        assert int(r[0]) in (0, 1) and int(r[1]) in (0, 1, 2) and int(r[8]) == 0
        assert 0.0 <= float(r[6]) <= float(r[7])
        assert 0 < int(r[5]) <= 300
