"""Multi-rank plumbing of the patch update: partition of an AMR patch table
across ranks and the two collectives the reference uses at rank boundaries.

The reference distributes patches with AMReX's DistributionMapping and
reduces the time step with MPI_Allreduce(MIN) (include/fub/solver/
SubcycleFineFirstSolver.hpp:100-112, DimensionalSplitLevelIntegrator.hpp:
240-242, src/ext/Mpi.cpp:55-58).  Here one process drives one GPU; with one
GPU per machine the runs are independent replicas, so these functions serve
the replica bench (slowest-rank timing) and the host-side partition, which
is exercised by gloo ranks on the CPU.
"""
from __future__ import annotations

import numpy as np


def morton_key(ix, iy, bits=21):
    """Interleaved bits of non-negative integer coordinates (Z order)."""
    ix = np.asarray(ix, dtype=np.uint64)
    iy = np.asarray(iy, dtype=np.uint64)
    key = np.zeros_like(ix)
    for b in range(bits):
        key |= ((ix >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b)
        key |= ((iy >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b + 1)
    return key


def patch_weights(hier, ghost=2):
    """Storage cells of every patch (interior plus halo), the work weight."""
    b = np.asarray(hier.boxes).reshape(-1, 4).astype(np.int64)
    return (b[:, 2] - b[:, 0] + 2 * ghost) * (b[:, 3] - b[:, 1] + 2 * ghost)


def morton_order(hier):
    """Patch indices sorted by the Z-order key of their centres, measured in
    cells of the finest level (so that refined regions stay together)."""
    b = np.asarray(hier.boxes).reshape(-1, 4).astype(np.int64)
    lv = np.asarray(hier.levels).astype(np.int64)
    shift = (hier.nlevels - 1) - lv
    cx = ((b[:, 0] + b[:, 2]) << shift) // 2
    cy = ((b[:, 1] + b[:, 3]) << shift) // 2
    return np.argsort(morton_key(cx, cy), kind="stable")


def partition(hier, nranks, ghost=2):
    """Contiguous runs of the Morton order with balanced storage weight:
    returns one array of patch indices per rank.  The heaviest rank carries
    at most the mean weight plus one patch's weight."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    order = morton_order(hier)
    w = patch_weights(hier, ghost)[order]
    cum = np.cumsum(w)
    total = int(cum[-1]) if len(cum) else 0
    # rank r takes the patches whose cumulative weight midpoint falls in
    # [r, r+1) * total / nranks
    mid = cum - w / 2.0
    owner = np.minimum((mid * nranks / max(total, 1)).astype(np.int64), nranks - 1)
    return [order[owner == r] for r in range(nranks)]


def allreduce_min(value: float, group=None) -> float:
    """MinAll of one double (src/ext/Mpi.cpp:55-58) over torch.distributed
    (gloo on the CPU, NCCL on GPUs); the identity without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    return float(t.item())


def slowest(ms: float, group=None) -> float:
    """The slowest rank's time (max over ranks), used for whole-job rates."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(ms)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
