"""Column sharding across ranks (one process per GPU).

Sediment columns are independent: the transport is vertical-only and the
rates are local, so the reference decomposes the grid into ESMF PETs with no
halo exchange (src/components/fabm_sediment_component.F90:382-387).  Here a
rank owns a contiguous range of grid columns, balanced by active layers, and
steps it with its own handle.  No data crosses ranks during a run; only the
scalar step statistics are reduced, once, at the end.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .model import ColumnSet


def partition(kact: np.ndarray, world: int) -> List[Tuple[int, int]]:
    """Contiguous column ranges [c0, c1), one per rank, with about equal
    sums of the per-column work ``kact`` (active layers, or any nonnegative
    weight; land columns count as nothing).  With more ranks than columns
    some ranges are empty; such a rank has nothing to step."""
    kact = np.asarray(kact, dtype=np.float64)
    ncol = kact.size
    if world < 1:
        raise ValueError("world must be >= 1")
    work = np.cumsum(kact)
    total = float(work[-1]) if ncol else 0.0
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        c = int(np.searchsorted(work, target, side="left")) + 1
        bounds.append(min(max(c, bounds[-1]), ncol))
    bounds.append(ncol)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def shard(cs: ColumnSet, rank: int, world: int) -> Tuple[ColumnSet, Tuple[int, int]]:
    """The rank's columns as their own 1 x n grid, and its column range."""
    c0, c1 = partition(cs.kact, world)[rank]
    return cs.subset(np.arange(c0, c1)), (c0, c1)


def shard_pelagic(pcs, rank: int, world: int):
    """The pelagic grid's share of one rank: a contiguous column range with
    about equal water cells, as its own 1 x n grid, and the range."""
    c0, c1 = partition(pcs.water().sum(axis=0), world)[rank]
    return pcs.subset(np.arange(c0, c1)), (c0, c1)


# A water cell's Run against a soil layer's coupling step on GB300: 1.22 ms
# per Run of 22.0 M water cells (pelagic_1024x1024) and 27.1 ms per step of
# 25.7 M active layers (uneven_1024x1024), i.e. 0.055 against 1.05 ns.
PEL_CELL_WEIGHT = 0.05


def shard_coupled(pcs, cs: ColumnSet, rank: int, world: int,
                  pel_weight: float = PEL_CELL_WEIGHT):
    """One rank's share of a coupled pelagic / soil grid (the same inum x
    jnum): the same contiguous column range of both, so each rank's
    cpl_pelagic_soil reads and writes only its own columns and no field
    crosses ranks.  The ranges balance the soil's active layers plus
    pel_weight times the water cells of each column.  Returns the pelagic
    and soil shards as their own 1 x n grids, and the range."""
    if pcs.ncol != cs.ncol:
        raise ValueError("the pelagic and soil grids differ in inum*jnum")
    work = np.asarray(cs.kact, dtype=np.float64) + pel_weight * pcs.water().sum(axis=0)
    c0, c1 = partition(work, world)[rank]
    cols = np.arange(c0, c1)
    return pcs.subset(cols), cs.subset(cols), (c0, c1)


_SUM = ("attempts", "accepted", "column_steps", "capped_columns", "nan_cells",
        "gpu_launches", "surrogate_columns", "capped_cells")
_MAX = ("max_col_attempts", "max_cell_attempts", "device_ms")


def reduce_stats(stats: Dict[str, float], group=None) -> Dict[str, float]:
    """Whole-grid statistics from every rank's sed_stats dict: sums of the
    counters, max of the per-column maxima and of the device time, min of the
    smallest substep (torch.distributed, any backend)."""
    import torch
    import torch.distributed as dist
    # nccl reduces device tensors, gloo host ones
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    keys = [k for k in _SUM if k in stats]
    s = torch.tensor([float(stats[k]) for k in keys], dtype=torch.float64, device=dev)
    mkeys = [k for k in _MAX if k in stats] or ["max_col_attempts"]
    mx = torch.tensor([float(stats.get(k, 0)) for k in mkeys], dtype=torch.float64, device=dev)
    mn = torch.tensor([float(stats.get("min_dt", np.inf))], dtype=torch.float64, device=dev)
    dist.all_reduce(s, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(mn, op=dist.ReduceOp.MIN, group=group)
    out = dict(stats)
    for k, v in zip(keys, s.tolist()):
        out[k] = int(v)
    for k, v in zip(mkeys, mx.tolist()):
        out[k] = float(v) if k == "device_ms" else int(v)
    out["min_dt"] = float(mn[0].item())
    return out
