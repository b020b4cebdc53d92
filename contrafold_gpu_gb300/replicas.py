"""Folding a task list on several GPUs: one process per GPU, no collective on
the data path.

Folds are independent, so a list of sequences is partitioned by estimated cost
(~ L^3: the bifurcation recurrences dominate) with longest-processing-time-first
assignment, each rank folds its own part on its own GPU, and the results are
gathered on the host (`torch.distributed.all_gather_object` -- gloo or NCCL,
once per call, outside the fold).

    import torch.distributed as dist
    from contrafold_gpu_gb300 import replicas
    dist.init_process_group("nccl")       # torchrun, one rank per GPU
    structs = replicas.fold_distributed(seqs, replicas.mea_folder(P, gamma=6.0), masks)
"""
from __future__ import annotations

import heapq
from typing import Callable, List, Optional, Sequence


def lpt_partition(lengths: Sequence[int], world: int) -> List[List[int]]:
    """Indices of `lengths` split into `world` parts of near-equal total L^3,
    longest first onto the least-loaded part; each part keeps ascending index
    order.  Deterministic (ties go to the lower rank)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(lengths)), key=lambda k: (-int(lengths[k]), k))
    heap = [(0, r) for r in range(world)]
    parts: List[List[int]] = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        parts[r].append(k)
        heapq.heappush(heap, (load + max(int(lengths[k]), 1) ** 3, r))
    return [sorted(p) for p in parts]


def fold_distributed(seqs: Sequence[str], fold: Callable[[List[str], Optional[list]], list],
                     masks: Optional[Sequence] = None, group=None) -> list:
    """Fold `seqs` across the ranks of `group` (the default process group; a
    single process when torch.distributed is not initialised).  `fold(part,
    part_masks)` folds one rank's part on that rank and returns one result per
    sequence; every rank returns the full result list in input order."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return list(fold(list(seqs), None if masks is None else list(masks)))
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    parts = lpt_partition([len(s) for s in seqs], world)
    mine = parts[rank]
    local = fold([seqs[k] for k in mine], None if masks is None else [masks[k] for k in mine]) if mine else []
    if len(local) != len(mine):
        raise RuntimeError("fold returned a wrong number of results")
    gathered: list = [None] * world
    dist.all_gather_object(gathered, (mine, list(local)), group=group)
    out: list = [None] * len(seqs)
    for idx, res in gathered:
        for k, v in zip(idx, res):
            out[k] = v
    return out


def mea_folder(P: dict, gamma: float = 6.0, device: Optional[int] = None):
    """A `fold` for fold_distributed: MEA structures on this rank's GPU (the
    local rank's device under torchrun)."""
    import os

    from .engine import Batch, Engine
    dev = int(os.environ.get("LOCAL_RANK", "0")) if device is None else device
    eng = Engine(P, device=dev)

    def fold(part, part_masks):
        return eng.mea(Batch(part, part_masks), gamma)

    return fold
