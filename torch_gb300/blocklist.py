"""Leaf-block lists across ranks.

PARAMESH hands each MPI rank a contiguous range of the Morton-ordered
(space-filling-curve) block list, and FLASH reduces the per-rank CFL limit
with MPI_AllReduce(MINLOC) (Driver_computeDt.F90:514-515). These are the
host-side pieces of the same scheme for one process per GPU over
torch.distributed: the Morton order of a block tree's leaves, the split of
that order into contiguous ranges of equal work, and the global dt minimum
with the rank and block that set it.
"""
from __future__ import annotations

import numpy as np


def _spread3(v: np.ndarray) -> np.ndarray:
    """Spread the low 21 bits of v so bit b lands on bit 3b."""
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
    v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
    v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
    return v


def morton_keys(tree: dict, blocks) -> np.ndarray:
    """Morton key of each block's lower corner in finest-level block units."""
    b = np.asarray(blocks)
    s = (int(tree["maxlevel"]) - np.asarray(tree["level"])[b]).astype(np.uint64)
    c = np.asarray(tree["coord"])[b].astype(np.uint64) << s[:, None]
    return _spread3(c[:, 0]) | (_spread3(c[:, 1]) << np.uint64(1)) | (_spread3(c[:, 2]) << np.uint64(2))


def morton_order(tree: dict, blocks=None) -> np.ndarray:
    """The leaves (or the given blocks) sorted along the Morton curve."""
    b = np.asarray(tree["leaf"] if blocks is None else blocks, np.int32)
    return b[np.argsort(morton_keys(tree, b), kind="stable")]


def split_blocks(order: np.ndarray, nranks: int, work=None) -> list:
    """Contiguous ranges of `order` with equal total work (one unit per
    block unless `work` gives per-block costs), one per rank."""
    order = np.asarray(order)
    w = np.ones(len(order)) if work is None else np.asarray(work, float)
    cum = np.concatenate([[0.0], np.cumsum(w)])
    cuts = [0]
    for r in range(1, nranks):
        cuts.append(int(np.searchsorted(cum, cum[-1] * r / nranks, side="left")))
    cuts.append(len(order))
    return [order[cuts[r]:cuts[r + 1]] for r in range(nranks)]


def global_dt(local_dt: float, local_block: int = -1, group=None):
    """(dt, rank, block): the minimum of every rank's CFL limit, the rank
    that holds it and that rank's limiting block (MPI_AllReduce MINLOC).
    Without an initialised process group it is the local value."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(local_dt), 0, int(local_block)
    rank = dist.get_rank(group)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(local_dt)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    dt = float(t.item())
    # lowest rank whose local value equals the minimum, and its block
    cand = torch.tensor([rank if float(local_dt) == dt else 1 << 30, int(local_block)], dtype=torch.int64,
                        device=dev)
    who = cand[:1].clone()
    dist.all_reduce(who, op=dist.ReduceOp.MIN, group=group)
    owner = int(who.item())
    blk = torch.tensor([int(local_block) if rank == owner else -(1 << 40)], dtype=torch.int64, device=dev)
    dist.all_reduce(blk, op=dist.ReduceOp.MAX, group=group)
    return dt, owner, int(blk.item())


def max_over_ranks(x: float, group=None) -> float:
    """The slowest rank's time (the bench's whole-job clock)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
