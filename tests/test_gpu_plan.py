"""Device-resident plans (cf_plan_*): results equal the host-buffer entry points,
with and without CUDA graph replay (cf_plan_set_graph), on every schedule."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(rng.integers(lo, hi + 1)))) for _ in range(n)]
    masks = [(rng.random(len(s)) < 0.1).astype(np.uint8) for s in seqs]
    return seqs, masks


def _device(torch, seqs, masks):
    dev = torch.device("cuda", 0)
    buf = np.frombuffer("".join(seqs).encode(), np.uint8).copy()
    mk = np.concatenate(masks).astype(np.uint8)
    offs = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(s) for s in seqs], out=offs[1:])
    return torch.from_numpy(buf).to(dev), torch.from_numpy(mk).to(dev), offs


@pytest.mark.parametrize("schedule", ["auto", "warp", "group", "cluster"])
def test_plan_matches_host_calls_with_and_without_graph(engine, schedule):
    torch = pytest.importorskip("torch")
    from contrafold_gpu_gb300.engine import CF_JOB_LOGZ, CF_JOB_LOGZ64, CF_JOB_MEA, CF_JOB_MFE, Batch, Plan
    engine.set_schedule(schedule)
    try:
        seqs, masks = _batch(7, 70, 10, 180)
        B = Batch(seqs, masks)
        d_seqs, d_mask, offs = _device(torch, seqs, masks)
        n, tot = len(seqs), int(offs[-1])
        stream = torch.cuda.Stream()
        want = {CF_JOB_MEA: engine.mea(B, 6.0), CF_JOB_MFE: engine.mfe(B),
                CF_JOB_LOGZ: engine.logz(B), CF_JOB_LOGZ64: engine.logz64(B)}
        for job, ref in want.items():
            for graph in (False, True):
                plan = Plan(engine, job, offs)
                plan.set_graph(graph)
                outs = []
                for _ in range(2):   # two outputs: the second run re-captures under graph replay
                    if job == CF_JOB_LOGZ:
                        out = torch.zeros(n, dtype=torch.float32, device="cuda")
                    elif job == CF_JOB_LOGZ64:
                        out = torch.zeros(n, dtype=torch.float64, device="cuda")
                    else:
                        out = torch.zeros(tot, dtype=torch.uint8, device="cuda")
                    for _ in range(2):   # repeated arguments: the graph is replayed
                        plan.run(d_seqs.data_ptr(), d_mask.data_ptr(), out.data_ptr(), 6.0, stream.cuda_stream)
                    plan.status()
                    torch.cuda.synchronize()
                    outs.append(out.cpu().numpy())
                assert plan.launches >= 1
                plan.close()
                for o in outs:
                    if job in (CF_JOB_MEA, CF_JOB_MFE):
                        s = o.tobytes().decode()
                        assert [s[offs[b]:offs[b + 1]] for b in range(n)] == ref, (job, graph)
                    else:
                        assert np.array_equal(o, np.asarray(ref)), (job, graph)
    finally:
        engine.set_schedule("auto")


def test_phase_timing_runs_the_per_phase_kernels(engine):
    """With phase timing on, a grouped MEA plan runs four per-phase kernels
    instead of the fused one; structures are identical and the phases timed."""
    torch = pytest.importorskip("torch")
    from contrafold_gpu_gb300.engine import CF_JOB_MEA, Batch, Plan
    engine.set_schedule("group")
    try:
        seqs, masks = _batch(11, 90, 30, 160)
        d_seqs, d_mask, offs = _device(torch, seqs, masks)
        tot = int(offs[-1])
        outs = {}
        for timing in (False, True):
            plan = Plan(engine, CF_JOB_MEA, offs)
            assert plan.schedule == "group"
            plan.set_timing(timing)
            out = torch.zeros(tot, dtype=torch.uint8, device="cuda")
            plan.run(d_seqs.data_ptr(), d_mask.data_ptr(), out.data_ptr(), 6.0, 0)
            plan.status()
            torch.cuda.synchronize()
            outs[timing] = out.cpu().numpy().tobytes()
            assert plan.launches == (4 if timing else 1)
            if timing:
                assert np.all(plan.phase_ms() > 0)
            plan.close()
        assert outs[False] == outs[True]
        assert outs[False].decode() == "".join(engine.mea(Batch(seqs, masks), 6.0))
    finally:
        engine.set_schedule("auto")


def test_auto_schedule_takes_cluster_for_small_long_batches(engine):
    """Automatic schedule: a few sequences of >= 512 nt fold on a cluster each;
    a larger batch of 300-nt sequences stays grouped."""
    from contrafold_gpu_gb300.engine import CF_JOB_LOGZ, CF_JOB_MEA, Plan
    engine.set_schedule("auto")
    for job in (CF_JOB_MEA, CF_JOB_LOGZ):
        plan = Plan(engine, job, np.array([0, 600, 1300], np.int64))
        assert plan.schedule == "cluster"
        plan.close()
    plan = Plan(engine, CF_JOB_MEA, np.arange(65, dtype=np.int64) * 300)
    assert plan.schedule == "group"
    plan.close()
