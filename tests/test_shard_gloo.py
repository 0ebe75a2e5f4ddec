"""The multi-rank path on CPU: two gloo ranks, each matching its root range
(with the oracle standing in for the GPU matcher, which needs a GPU), must
reproduce the full count and the full table exactly; the work-weighted root
split covers every root once and balances the estimated work on R-MAT."""
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


def test_weighted_root_ranges_cover_and_balance_on_rmat():
    import numpy as np

    from forkmatch_gb300 import synth as S
    G = S.rmat(14, 120000, 11, 4)
    src, _, _ = G.directed()
    w = shard.root_work_weights(src, G.V)
    for world in (1, 2, 3, 4, 8, 16):
        rs = shard.root_ranges_weighted(w, world)
        assert len(rs) == world and rs[0][0] == 0 and rs[-1][1] == G.V
        assert all(rs[i][1] == rs[i + 1][0] for i in range(world - 1))
        assert all(b <= e for b, e in rs)
        covered = np.zeros(G.V, dtype=np.int64)
        for b, e in rs:
            covered[b:e] += 1
        assert (covered == 1).all()
        loads = np.array([w[b:e].sum() for b, e in rs])
        assert loads.max() <= w.sum() / world + w.max() + 1e-6
    # equal-length ranges put the hubs' work on few ranks; the weighted split does not
    eq = [w[b:e].sum() for b, e in shard.root_ranges(G.V, 8)]
    wt = [w[b:e].sum() for b, e in shard.root_ranges_weighted(w, 8)]
    assert max(wt) <= max(eq)


def test_split_queries_balances_and_covers():
    costs = [100, 1, 1, 50, 50, 3, 7, 7, 90, 10]
    for world in (1, 2, 3, 4, 16):
        parts = shard.split_queries(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        if world <= len(costs):
            assert max(loads) <= sum(costs) / world + max(costs)


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
    b, e = shard.root_ranges_weighted(shard.root_work_weights(src, G.V), world)[rank]
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


def _batch_rank_main(rank, world, port, result_q):
    import torch.distributed as dist

    from forkmatch_gb300 import synth as S
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    G = S.erdos_renyi(300, 1500, seed=8, n_elabels=2)
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, 3, src, dst, lab)
    queries = [S.query_cycle(4, [1, 2, 1, 2]), S.query_path(4, [1, 1, 2]), S.query_cycle(3, [1, 1, 2]),
               S.query_star(4, [1, 2, 2]), S.query_path(3, [2, 2]), S.query_clique(4, [1, 2])]
    plans = [O.plan(qq.to_g_text(), enumerate_aut=0) for qq in queries]
    costs = [len(qq.edges) for qq in queries]
    mine = shard.split_queries(costs, world)[rank]
    counts = [O.match(og, plans[i], threads=1)[0] for i in mine]
    total = shard.merge_query_counts(dist, len(queries), mine, counts)
    if rank == 0:
        full = [O.match(og, p, threads=1)[0] for p in plans]
        result_q.put((total == full, total, full))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_split_a_batch_by_query():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_batch_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    ok, total, full = q.get(timeout=10)
    assert ok, (total, full)
