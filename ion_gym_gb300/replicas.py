"""Several GPUs of one node, one process per GPU.

The field solve shards without a data-path collective: the bases of one
deck are independent solves over the same metal union, and decks are
independent of each other, so each rank solves its own share and keeps its
results.  The only communication is for timing: a barrier around the timed
region and the maximum of the ranks' elapsed times (whole-job throughput =
the units all ranks processed / that maximum).  Ranks, world size and the
rendezvous come from the torchrun environment (RANK, WORLD_SIZE,
LOCAL_RANK, MASTER_ADDR, MASTER_PORT).
"""
import os


def world():
    """(world size, rank, local rank) from the environment; (1, 0, 0)
    outside torchrun."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend=None, device=None):
    """Join the process group when the world has more than one rank:
    NCCL for CUDA ranks (bound to `device`), gloo otherwise."""
    ws, _, _ = world()
    if ws <= 1:
        return False
    import torch.distributed as dist
    if dist.is_initialized():
        return True
    if backend is None:
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl" and device is not None:
        dist.init_process_group(backend, device_id=device)
    else:
        dist.init_process_group(backend)
    return True


def _active():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier():
    dist = _active()
    if dist is not None:
        dist.barrier()


def _reduce(x, op, device):
    dist = _active()
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, device="cpu"):
    """The largest value of x over the ranks (x itself with one rank)."""
    dist = _active()
    return x if dist is None else _reduce(x, dist.ReduceOp.MAX, device)


def sum_over_ranks(x, device="cpu"):
    dist = _active()
    return x if dist is None else _reduce(x, dist.ReduceOp.SUM, device)


def throughput(units, elapsed, device="cpu"):
    """Whole-job throughput: the units every rank processed divided by the
    slowest rank's elapsed time."""
    return sum_over_ranks(units, device) / max_over_ranks(elapsed, device)


def shard(keys, rank=None, size=None):
    """This rank's share of a set of independent problems: the sorted keys
    dealt round-robin, so shares differ in size by at most one and every
    key belongs to exactly one rank."""
    if rank is None or size is None:
        size, rank, _ = world()
    return sorted(keys)[rank::size]


def solve_bases_sharded(masks, rank=None, size=None, **kwargs):
    """This rank's bases of a deck through the basis door
    (multigrid3d.solve_bases_mg with `only` = the rank's share); the
    returned dict holds only those bases.  Each basis is bit-identical to a
    single-rank solve."""
    from ion_gym_gb300.physics import multigrid3d as MG
    mine = set(shard(masks.keys(), rank, size))
    only = kwargs.pop("only", None)
    if only is not None:
        mine &= set(only)
    return MG.solve_bases_mg(masks, only=mine, **kwargs)


def solve_bases_mixed_sharded(masks, spec=None, root=None, rank=None,
                              size=None, v_basis=1e4, accuracy=1e-9, **kwargs):
    """The mixed-precision basis batch of one deck, sharded over the ranks:
    each rank solves its round-robin share of the bases in its own batched
    session (physics.mixed.solve_bases_mixed; `only` narrows the set) and
    returns {index: phi float64 at v_basis} for that share.

    With `spec`, the ranks' results also become one cache entry in the
    reference's 3-D layout (build_stl3d.py:919-924: float32 unit bases
    basis_<i> and the uint8 labels): each rank stages its unit bases as .npy
    files in a folder beside the cache (the gather goes through the shared
    disk of the node, not through the process group), and after a barrier
    rank 0 stores the entry from them (fa_cache.store, published
    atomically) and removes the staging folder.  Every rank returns
    (its bases, the entry key) then."""
    import numpy as np
    from ion_gym_gb300.physics import mixed
    from ion_gym_gb300.io import fa_cache
    if rank is None or size is None:
        size, rank, _ = world()
    mine = set(shard(masks.keys(), rank, size))
    only = kwargs.pop("only", None)
    if only is not None:
        mine &= set(only)
    out = mixed.solve_bases_mixed(masks, v_basis=v_basis, accuracy=accuracy,
                                  only=mine, **kwargs) if mine else {}
    if spec is None:
        return out
    key = fa_cache.spec_key(spec)
    base = os.path.expanduser(fa_cache._root(root))
    stage = os.path.join(base, f".{key}.shards")
    os.makedirs(stage, exist_ok=True)
    for i, phi in out.items():
        unit = (np.asarray(phi) / v_basis).astype(np.float32)
        tmp = os.path.join(stage, f".basis_{i}.{rank}.npy")
        np.save(tmp, unit)
        os.replace(tmp, os.path.join(stage, f"basis_{i}.npy"))
    barrier()
    if rank == 0:
        want = sorted(i for i in masks if only is None or i in only)
        arrays = {f"basis_{i}": np.load(os.path.join(stage, f"basis_{i}.npy"),
                                        mmap_mode="r") for i in want}
        shape = np.asarray(next(iter(masks.values()))).shape
        lab = np.zeros(shape, np.uint8)
        for i, m in masks.items():
            lab[np.asarray(m, bool)] = i
        arrays["labels"] = lab
        fa_cache.store(spec, arrays, root=root)
        del arrays
        import shutil
        shutil.rmtree(stage, ignore_errors=True)
    barrier()
    return out, key
