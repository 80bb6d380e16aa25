"""Data-parallel X^T X assembly over several ranks.

Structures are independent, so a fit shards them: each rank builds the rows of
its structures and its partial X^T X, X^T y, y^T y and energy-row column sums,
and one sum all-reduce combines them; the ridge solve then runs on every rank
(or on one, with the coefficients broadcast).  This is the data-parallel form
of calc_xtx_xty (src/pypolymlp/mlp_dev/core/data_sequential.py:25-152), whose
sums over structure batches are order-independent up to rounding.

The reduction goes through torch.distributed (NCCL for CUDA tensors, gloo on
the host), with the partial results as FP64 tensors.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def shard_ranges(n_rows_per_structure: Sequence[int], world: int) -> List[Tuple[int, int]]:
    """Contiguous structure ranges, one per rank, balanced by cumulative row count."""
    rows = np.asarray(n_rows_per_structure, dtype=np.int64)
    n = len(rows)
    if world < 1:
        raise ValueError("world must be >= 1")
    cum = np.concatenate([[0], np.cumsum(rows)])
    total = cum[-1]
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        bounds.append(int(np.searchsorted(cum, target, side="left")))
    bounds.append(n)
    bounds = np.maximum.accumulate(np.clip(bounds, 0, n))
    return [(int(bounds[r]), int(bounds[r + 1])) for r in range(world)]


def structure_rows(n_atoms: Sequence[int], include_force: bool = True) -> np.ndarray:
    """Rows each structure contributes: 1 energy, and 6 stress + 3N force rows with forces."""
    n = np.asarray(n_atoms, dtype=np.int64)
    return 1 + (6 + 3 * n if include_force else 0 * n)


def allreduce_sums(arrays: Sequence[np.ndarray], device=None) -> List[np.ndarray]:
    """Sum FP64 host arrays over all ranks of the default process group (in place
    semantics: returns the reduced arrays).  device: where the collective runs
    (None = host tensors, for gloo; 'cuda' for NCCL)."""
    import torch
    import torch.distributed as dist

    flat = np.concatenate([np.asarray(a, dtype=np.float64).ravel() for a in arrays])
    t = torch.from_numpy(flat)
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    flat = t.cpu().numpy()
    out, pos = [], 0
    for a in arrays:
        a = np.asarray(a)
        out.append(flat[pos:pos + a.size].reshape(a.shape))
        pos += a.size
    return out


def allreduce_gram(result, device=None):
    """All-reduce the tuple returned by GramAccumulator.result():
    (xtx, xty, yty, xe_sum, xe_sq, n_rows)."""
    xtx, xty, yty, xe_sum, xe_sq, n_rows = result
    r = allreduce_sums([xtx, xty, np.array([yty]), xe_sum, xe_sq, np.array([float(n_rows)])], device)
    return r[0], r[1], float(r[2][0]), r[3], r[4], int(round(r[5][0]))
