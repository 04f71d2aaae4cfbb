"""The multi-GPU path on CPU: two gloo ranks (127.0.0.1) exercise the
replica logic the benchmark and the sharded basis door use -- the barrier,
the slowest rank's time, whole-job throughput, and the dealing of
independent bases so every basis belongs to exactly one rank, and the
sharded mixed-precision batch whose ranks' bases rank 0 assembles into one
cache entry.  No GPU: the basis door and the mixed batch are replaced by
recorders of what each rank was asked to solve."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, size, port, q, cache_root):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(size), LOCAL_RANK=str(rank))
    import numpy as np
    from ion_gym_gb300 import replicas
    from ion_gym_gb300.physics import multigrid3d as MG
    assert replicas.init("gloo")
    replicas.barrier()
    el = 1.0 + rank                       # rank 1 is the slow one
    units = 3 * (rank + 1)
    got = {"max": replicas.max_over_ranks(el),
           "sum": replicas.sum_over_ranks(units),
           "thr": replicas.throughput(units, el)}
    asked = []

    def fake_door(masks, only=None, **kw):
        asked.append(sorted(only))
        return {i: np.full(1, float(i)) for i in sorted(only)}

    MG.solve_bases_mg = fake_door
    masks = {k: None for k in (4, 1, 7, 2, 9)}
    out = replicas.solve_bases_sharded(masks, tol=1e-5)
    got["mine"] = sorted(out)
    got["asked"] = asked
    got["shard_default"] = replicas.shard(masks.keys())
    # the mixed batch, sharded, assembled into one cache entry by rank 0
    from ion_gym_gb300.physics import mixed
    solved = []

    def fake_mixed(masks, v_basis=1e4, accuracy=1e-9, only=None, **kw):
        solved.append(sorted(only))
        return {i: np.full((3, 4, 5), v_basis * i / 10.0) for i in sorted(only)}

    mixed.solve_bases_mixed = fake_mixed
    deck = {}
    for i in (4, 1, 7, 2, 9):
        m = np.zeros((3, 4, 5), bool)
        m[i % 3, i % 4, i % 5] = True
        deck[i] = m
    spec = {"name": "sharded deck", "geometry": {"n": 5}}
    bases, key = replicas.solve_bases_mixed_sharded(deck, spec=spec,
                                                     root=cache_root)
    got["mixed_mine"] = sorted(bases)
    got["mixed_solved"] = solved
    got["key"] = key
    replicas.barrier()
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((rank, got))


def test_two_gloo_ranks_share_the_work(tmp_path):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    root = str(tmp_path / "cache")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q, root))
             for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert res[r]["max"] == 2.0
        assert res[r]["sum"] == 9.0
        assert res[r]["thr"] == pytest.approx(4.5)
    a, b = res[0]["mine"], res[1]["mine"]
    assert a == [1, 4, 9] and b == [2, 7]
    assert sorted(a + b) == [1, 2, 4, 7, 9] and not set(a) & set(b)
    assert res[0]["asked"] == [a] and res[1]["asked"] == [b]
    assert res[0]["shard_default"] == a and res[1]["shard_default"] == b
    # sharded mixed batch: each rank solved its share once; one entry holds
    # every basis (float32 unit bases) and the labels
    assert res[0]["mixed_solved"] == [a] and res[1]["mixed_solved"] == [b]
    assert res[0]["mixed_mine"] == a and res[1]["mixed_mine"] == b
    assert res[0]["key"] == res[1]["key"]
    import numpy as np
    from ion_gym_gb300.io import fa_cache
    arrs, meta = fa_cache.load(res[0]["key"], root=root)
    assert sorted(arrs) == ["basis_1", "basis_2", "basis_4", "basis_7",
                            "basis_9", "labels"]
    for i in (1, 2, 4, 7, 9):
        assert arrs[f"basis_{i}"].dtype == np.float32
        assert np.all(arrs[f"basis_{i}"] == np.float32(i / 10.0))
        assert arrs["labels"][i % 3, i % 4, i % 5] == i
    assert [n for n in os.listdir(root) if n.startswith(".")] == []


def test_one_rank_is_the_identity():
    from ion_gym_gb300 import replicas
    assert replicas.world()[0] >= 1
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.throughput(10, 2.0) == 5.0
    assert replicas.shard([3, 1, 2], 0, 1) == [1, 2, 3]
    assert replicas.shard(range(10), 2, 3) == [2, 5, 8]
