"""The multi-rank path on CPU: two gloo ranks, each matching its root range
(with the oracle standing in for the GPU matcher), must reproduce the full
count and the full table exactly."""
import os
import socket

import pytest

from forkmatch_gb300 import shard


def test_root_ranges_partition():
    for V in (0, 1, 7, 1000, 1 << 20):
        for world in (1, 2, 3, 8):
            rs = shard.root_ranges(V, world)
            assert len(rs) == world and rs[0][0] == 0 and rs[-1][1] == V
            assert all(rs[i][1] == rs[i + 1][0] for i in range(world - 1))
            assert all(b <= e for b, e in rs)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, result_q):
    import torch.distributed as dist

    from forkmatch_gb300 import synth as S
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    G = S.erdos_renyi(400, 2400, seed=7, n_elabels=2)
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, 3, src, dst, lab)
    queries = [S.query_cycle(4, [1, 2, 1, 2]), S.query_path(4, [1, 1, 2]), S.query_cycle(3, [1, 1, 2])]
    b, e = shard.root_ranges(G.V, world)[rank]
    counts, tables = [], []
    for qq in queries:
        p = O.plan(qq.to_g_text(), enumerate_aut=0)
        c, rows, _ = O.match(og, p, roots=(b, e), table=True, threads=1)
        counts.append(c)
        tables.append([tuple(r) for r in rows.tolist()])
    total = shard.reduce_counts(dist, counts)
    merged = [shard.gather_tables(dist, t) for t in tables]
    if rank == 0:
        full = []
        for qq in queries:
            p = O.plan(qq.to_g_text(), enumerate_aut=0)
            c, rows, _ = O.match(og, p, table=True, threads=1)
            full.append((c, sorted(tuple(r) for r in rows.tolist())))
        ok = all(t == f[0] for t, f in zip(total, full)) and all(sorted(m) == f[1] for m, f in zip(merged, full))
        result_q.put((ok, total, [f[0] for f in full]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_full_result():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    ok, total, full = q.get(timeout=10)
    assert ok, (total, full)
