"""Host-side sharding for running the pipeline as independent replicas, one
process per GPU. The caller supplies the process group (any object with the
torch.distributed-style get_rank / get_world_size / gather_object /
all_gather_object calls, e.g. a gloo group); only host objects travel through
it, and this module imports nothing but numpy.

The path has no exchange step: pixels, film row slabs, sample passes and whole
scenes are independent. A multi-GPU job therefore splits its units across
ranks with `shard`, renders them with its own context, and assembles results
on the host: film row slabs by `gather_rows` (concatenation on rank 0) and the
differentiable estimator's gradient by `allreduce_sum` (a sum of per-rank
gradients of disjoint pixel sets)."""
import numpy as np


def shard(n_units, world, rank):
    """Contiguous, balanced [start, end) range of n_units for `rank` of `world`."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_scenes(costs, world):
    """Scenes to ranks, largest estimated cost first onto the least loaded rank;
    returns one list of scene indices per rank (each list in ascending order)."""
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for k in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda j: (load[j], j))
        out[r].append(k)
        load[r] += costs[k]
    return [sorted(o) for o in out]


def gather_rows(local, total_rows, dist, dst=0):
    """Concatenate every rank's row slab (shape (rows_r, ...), ranks in order) on
    `dst`; returns the full array there and None elsewhere."""
    parts = [None] * dist.get_world_size() if dist.get_rank() == dst else None
    dist.gather_object(np.ascontiguousarray(local), parts, dst=dst)
    if dist.get_rank() != dst:
        return None
    full = np.concatenate(parts, axis=0)
    if full.shape[0] != total_rows:
        raise ValueError("gathered %d rows, expected %d" % (full.shape[0], total_rows))
    return full


def allreduce_sum(arr, dist):
    """Element-wise sum over ranks of a float array, on the host: every rank
    receives every rank's array and adds them in rank order in float64, so
    all ranks hold the same bits."""
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, np.ascontiguousarray(arr))
    acc = np.zeros(np.shape(arr), np.float64)
    for p in parts:
        acc += np.asarray(p, np.float64)
    return acc.astype(np.asarray(arr).dtype)
