"""Scene sharding across ranks (one process per GPU, no data-path collective).

Independent scenes are the only unit this path shards: one scene's step
would need particle halos and migration between GPUs, which is not built.
A batched workload's scenes are split across ranks by a greedy
longest-processing-time assignment on each scene's device footprint, every
rank steps its own scenes as one batched sim, and the only collective is the
reduction of the per-rank timings (max over ranks) after the timed region.
"""
from __future__ import annotations

import heapq

# Device bytes per unit, following the buffers cwa_create allocates:
# particles: P, V, ID (x2, ping-pong), F, RP, EX, key/slot/list, KS, nbr_cnt,
# the 64-code neighbour list, the two force gather records and a 64-byte
# staging record; grid cells: count + start + scan workspace; wave cells:
# three height buffers (+ the spare for the blocked advance) and the int64
# deposits.
BYTES_PER_PARTICLE = 2 * (16 + 16 + 4) + 16 + 8 + 8 + 12 + 4 + 4 + 64 * 2 + 32 + 64
BYTES_PER_CELL = 4 + 4 + 1
BYTES_PER_WAVE_CELL = 4 * 4 + 8


def grid_cells(desc) -> int:
    """Cells of the scene's sort grid (cwa_grid_dims; host-only call)."""
    import ctypes as C

    from . import _abi

    dims = (C.c_int32 * 3)()
    st = _abi.load().cwa_grid_dims(C.byref(desc), dims)
    if st != 0:
        raise _abi.CwaError(st, "cwa_grid_dims")
    return int(dims[0]) * int(dims[1]) * int(dims[2])


def scene_bytes(desc, grid_cells: int) -> int:
    """Approximate device footprint of one scene."""
    return (BYTES_PER_PARTICLE * int(desc.n_particles) + BYTES_PER_CELL * int(grid_cells)
            + BYTES_PER_WAVE_CELL * int(desc.wave_nx) * int(desc.wave_nz))


def assign(weights: list[int], world: int) -> list[list[int]]:
    """Split item indices over `world` ranks, heaviest first onto the least
    loaded rank (ties: lower rank, then lower index).  Deterministic, so every
    rank computes the same assignment without communicating.  Each rank's
    list is in ascending index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(weights)), key=lambda k: (-int(weights[k]), k))
    heap = [(0, r) for r in range(world)]
    out: list[list[int]] = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        out[r].append(k)
        heapq.heappush(heap, (load + int(weights[k]), r))
    return [sorted(x) for x in out]


def loads(weights: list[int], parts: list[list[int]]) -> list[int]:
    return [sum(int(weights[k]) for k in p) for p in parts]


def shard_scenes(workload, rank: int, world: int):
    """The scenes of `workload` that `rank` steps, as (indices, scenes)."""
    w = [scene_bytes(s.desc, grid_cells(s.desc)) for s in workload.scenes]
    mine = assign(w, world)[rank]
    return mine, [workload.scenes[k] for k in mine]


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank float over the default process group (gloo or nccl);
    the value itself when no group is initialised."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
