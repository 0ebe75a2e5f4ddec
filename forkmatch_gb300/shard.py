"""Sharding the search over several GPUs (one process per GPU).

Every subtree of the search is independent and the depth-0 roots partition it
(the reference already splits the vertex range across blocks,
src/smsm.cu:803-811).  Each rank holds a replica of the data graph and matches
the roots of its own range; the only exchange is a sum of per-query uint64
counts and, in table mode, a concatenation of the row blocks.  A batch can
instead be split by query (split_queries): each rank matches whole queries.
No collective runs on the data path.
"""


def root_ranges(V, world):
    """Equal contiguous root ranges [b, e), one per rank, covering [0, V)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    return [(V * r // world, V * (r + 1) // world) for r in range(world)]


def root_work_weights(src, V):
    """Estimated search work of each root vertex: d(v)^2 + 1, where d(v) is its
    number of e-lines (the partial matches two levels below a root grow with
    the square of its degree; the 1 charges the root lookup itself)."""
    import numpy as np
    d = np.bincount(np.asarray(src, dtype=np.int64), minlength=V).astype(np.float64)
    return d * d + 1.0


def root_ranges_weighted(weights, world):
    """Contiguous root ranges [b, e), one per rank, covering [0, len(weights)),
    cut where the prefix sum of the per-root work estimate crosses r/world of
    the total.  On R-MAT-like graphs, where a few hubs hold most of the work,
    equal-length ranges leave one rank with the hubs; these ranges give every
    rank about the same estimated work (each within one root's weight of
    total/world)."""
    import numpy as np
    if world < 1:
        raise ValueError("world must be >= 1")
    w = np.asarray(weights, dtype=np.float64)
    V = len(w)
    if V == 0:
        return [(0, 0)] * world
    c = np.cumsum(w)
    total = c[-1]
    cuts = [0]
    for r in range(1, world):
        # first root whose inclusive prefix reaches r/world of the work
        cuts.append(int(min(V, max(cuts[-1], np.searchsorted(c, total * r / world, side="left") + 1))))
    cuts.append(V)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def split_queries(costs, world):
    """Assign the queries of a batch to ranks: greedy longest-processing-time
    on an estimated cost per query (e.g. its recorded count or plain time).
    Returns, per rank, the ascending list of query indices it matches.  Every
    query goes to exactly one rank; each rank then runs its queries as one
    batch over its graph replica, and only the per-query counts (and tables)
    are exchanged."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        r = min(range(world), key=lambda r: (load[r], r))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


def merge_query_counts(dist, n, mine, counts):
    """Per-query counts of a query-sharded batch: rank r matched the queries
    `mine` with results `counts`; returns all n counts on every rank."""
    full = [0] * n
    for i, c in zip(mine, counts):
        full[i] = int(c)
    return reduce_counts(dist, full)


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
