"""Sample sharding across GPUs (one process per GPU).

Samples are independent rows of the recurrence, so a batch is split into
contiguous row ranges, every rank holds a full copy of the weights and runs
its own engine, and the only exchange is the final gather of the per-rank
category ids, shifted by each rank's row offset (no collective inside the
layer loop).  The reference has no multi-GPU path (its BF engine notes it
partitions inputs per GPU without communication, src/SDGC/BF/BF.hpp:11-13).
"""
import numpy as np


def shard_range(total_rows, world, rank):
    """Contiguous [offset, offset + count) rows of `rank`; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world or total_rows < 0:
        raise ValueError("bad shard arguments")
    base, extra = divmod(total_rows, world)
    offset = rank * base + min(rank, extra)
    count = base + (1 if rank < extra else 0)
    return offset, count


def gather_categories(local_ids, offset, group=None):
    """Global sorted survivor ids from every rank's local ids (torch.distributed)."""
    import torch.distributed as dist
    local = (np.asarray(local_ids, dtype=np.int64) + int(offset)).tolist()
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    out = np.array(sorted(i for p in parts for i in p), dtype=np.int64)
    return out


def run_shard(engine, inputs_fn, total_rows, rank, world, group=None):
    """Runs this rank's shard through `engine` and gathers the global category set.

    inputs_fn(offset, count) returns the rank's rows (count x N float32).
    """
    offset, count = shard_range(total_rows, world, rank)
    if count > 0:
        _, ids = engine.infer(inputs_fn(offset, count))
    else:
        ids = np.zeros(0, np.int32)
    return gather_categories(ids, offset, group)
