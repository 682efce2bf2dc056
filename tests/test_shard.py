"""Scene sharding host logic (coupledwateranimation_gb300/shard.py) on CPU:
the greedy assignment, and world_size-2 gloo process groups that split a
batched workload, reduce timings over ranks, and see a failed rank as an
error rather than a hang."""
from __future__ import annotations

import datetime
import multiprocessing as mp
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_assign_covers_and_balances():
    from coupledwateranimation_gb300 import shard

    rng = np.random.default_rng(0)
    w = rng.integers(1, 10_000, 257).tolist()
    for world in (1, 2, 3, 8):
        parts = shard.assign(w, world)
        assert sorted(k for p in parts for k in p) == list(range(len(w)))
        assert all(p == sorted(p) for p in parts)
        loads = shard.loads(w, parts)
        # list scheduling bound: makespan <= mean load + (1 - 1/m) * heaviest item
        assert max(loads) <= sum(w) / world + (1 - 1 / world) * max(w)
        assert parts == shard.assign(w, world)  # deterministic: ranks agree without talking


def test_assign_edge_cases():
    from coupledwateranimation_gb300 import shard

    assert shard.assign([], 3) == [[], [], []]
    assert shard.assign([5], 2) == [[0], []]
    assert shard.assign([1, 1, 1, 1], 4) == [[0], [1], [2], [3]]
    with pytest.raises(ValueError):
        shard.assign([1], 0)


def test_scene_bytes_grows_with_scene(lib):
    from coupledwateranimation_gb300 import scenes, shard

    a = scenes.dam_break((8, 8, 8), 0.02, (64, 64), seed=1)
    b = scenes.dam_break((16, 16, 16), 0.02, (256, 256), seed=1)
    ca, cb = shard.grid_cells(a.desc), shard.grid_cells(b.desc)
    assert ca > 0 and cb >= ca
    assert shard.scene_bytes(b.desc, cb) > shard.scene_bytes(a.desc, ca)


def _small_workload():
    from coupledwateranimation_gb300 import scenes

    sc = [scenes.dam_break((4 + k % 5, 6, 4 + k % 3), 0.02, (32 * (1 + k % 3), 32), seed=100 + k)
          for k in range(13)]
    return scenes.Workload("13 small scenes", sc, 1)


def _rank_main(rank: int, world: int, port: int, mode: str, q) -> None:
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    from coupledwateranimation_gb300 import shard

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    try:
        if mode == "fail" and rank == 1:
            raise RuntimeError("rank 1 fails before the timing reduction")
        wl = _small_workload()
        mine, _ = shard.shard_scenes(wl, rank, world)
        got = [None] * world
        dist.all_gather_object(got, mine)
        mx = shard.max_over_ranks(1.5 + rank)
        sm = shard.sum_over_ranks(float(len(mine)))
        q.put((rank, "ok", got, mx, sm))
    except Exception as e:  # noqa: BLE001 (reported to the parent)
        q.put((rank, "error", repr(e), None, None))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:  # noqa: BLE001
            pass


def _run(world: int, mode: str, timeout: float = 90.0):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, mode, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    try:
        for _ in range(world):
            r, status, a, b, c = q.get(timeout=timeout)
            out[r] = (status, a, b, c)
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    return out


def test_gloo_two_ranks_shard_and_reduce(lib):
    out = _run(2, "ok")
    assert out[0][0] == "ok" and out[1][0] == "ok", out
    parts0, parts1 = out[0][1], out[1][1]
    assert parts0 == parts1  # every rank sees the same assignment
    flat = sorted(k for p in parts0 for k in p)
    assert flat == list(range(13))
    assert out[0][2] == out[1][2] == 2.5  # max over ranks of 1.5 + rank
    assert out[0][3] == out[1][3] == 13.0


def test_gloo_failed_rank_is_an_error_not_a_hang(lib):
    out = _run(2, "fail")
    assert out[1][0] == "error"
    # rank 0 learns of the failure from its collective (peer gone or timeout)
    assert out[0][0] == "error", out[0]
