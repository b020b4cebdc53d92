"""Multi-GPU replicas, host side: LPT partition by L^3 and the gather of
fold_distributed, run as two gloo ranks on CPU with an injected fold."""
import os
import socket

import numpy as np
import pytest

from contrafold_gpu_gb300 import replicas


def test_lpt_partition_balances_cost_and_covers_every_index():
    rng = np.random.default_rng(0)
    lengths = list(rng.integers(40, 401, 500))
    for world in (1, 2, 3, 8):
        parts = replicas.lpt_partition(lengths, world)
        assert sorted(k for p in parts for k in p) == list(range(len(lengths)))
        loads = [sum(int(lengths[k]) ** 3 for k in p) for p in parts]
        # LPT bound: the heaviest part exceeds the mean by at most the largest job
        assert max(loads) - sum(loads) / world <= max(int(x) for x in lengths) ** 3
    assert replicas.lpt_partition([], 2) == [[], []]
    assert replicas.lpt_partition([5, 5], 2) == [[0], [1]]
    with pytest.raises(ValueError):
        replicas.lpt_partition([1], 0)


def test_fold_distributed_single_process():
    seqs = ["ACGU", "GGGGAAAACCCC", ""]
    assert replicas.fold_distributed(seqs, lambda part, m: [len(s) for s in part]) == [4, 12, 0]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, seqs, masks, queue):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seen = []

        def fold(part, part_masks):
            seen.extend(part)
            return [f"{len(s)}:{int(sum(m)) if m is not None else -1}" for s, m in zip(part, part_masks)]

        out = replicas.fold_distributed(seqs, fold, masks)
        queue.put((rank, out, seen))
    finally:
        dist.destroy_process_group()


def test_fold_distributed_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    rng = np.random.default_rng(1)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(L))) for L in rng.integers(1, 60, 37)]
    masks = [(rng.random(len(s)) < 0.2).astype(int).tolist() for s in seqs]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, seqs, masks, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = [f"{len(s)}:{sum(m)}" for s, m in zip(seqs, masks)]
    parts = replicas.lpt_partition([len(s) for s in seqs], 2)
    for rank, out, seen in res:
        assert out == want                                   # every rank gets the full, ordered result
        assert seen == [seqs[k] for k in parts[rank]]        # and folded only its own part


@pytest.mark.gpu
def test_mea_folder_matches_engine(engine, P):
    from contrafold_gpu_gb300.engine import Batch
    rng = np.random.default_rng(2)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(L))) for L in rng.integers(20, 150, 25)]
    assert replicas.fold_distributed(seqs, replicas.mea_folder(P, 6.0)) == engine.mea(Batch(seqs), 6.0)
