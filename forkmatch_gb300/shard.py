"""Sharding the search over several GPUs (one process per GPU).

Every subtree of the search is independent and the depth-0 roots partition it
(the reference already splits the vertex range across blocks,
src/smsm.cu:803-811).  Each rank holds a replica of the data graph and matches
the roots of its own range; the only exchange is a sum of per-query uint64
counts and, in table mode, a concatenation of the row blocks.  No collective
runs on the data path.
"""


def root_ranges(V, world):
    """Equal contiguous root ranges [b, e), one per rank, covering [0, V)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    return [(V * r // world, V * (r + 1) // world) for r in range(world)]


def reduce_counts(dist, counts):
    """Sum per-query counts over ranks (torch.distributed, any backend)."""
    import torch
    t = torch.tensor([int(c) for c in counts], dtype=torch.int64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t)
    return [int(x) for x in t.cpu().tolist()]


def gather_tables(dist, rows):
    """Concatenate every rank's table rows (list of rows) on every rank."""
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, rows)
    merged = []
    for part in out:
        merged.extend(part)
    return merged
