"""Batched matching (fm_batch_*): every query's count and table equal the
one-query-at-a-time results (fm_match) and the oracle, alone and in the mix,
on the first (captured) run and on graph replays, under forced level deferral,
after autotuning, and on the fallback path (duplicate e-lines, q == 1)."""
import numpy as np
import pytest

import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sorted(a):
    a = np.asarray(a, dtype=np.uint32)
    return a[np.lexsort(a.T[::-1])] if a.size else a


def _mix(G, rng, n=24):
    qs = [S.query_path(2, [1]), S.query_path(3, [1, 2]), S.query_cycle(3, [1, 1, 2]), S.query_cycle(4, [1, 2, 1, 2]),
          S.query_star(4, [1, 2, 2]), S.query_clique(4, [1, 2]), S.query_path(6, [1, 2, 1, 2, 1]),
          S.query_cycle(6, [1, 2, 1, 2, 1, 2])]
    while len(qs) < n:
        k = int(rng.integers(3, 9))
        q = S.query_random_walk(G, k, rng, tree=bool(len(qs) % 3 == 0), bias=1.0)
        if q is not None:
            qs.append(q)
    return qs


@pytest.fixture(scope="module")
def env():
    from forkmatch_gb300 import build
    build.build()
    ctx = fm.Context(prealloc_bytes=3 << 30, soln_prealloc_bytes=1 << 30, output_prealloc_bytes=1 << 30,
                     bank_rows=1024)
    G = S.erdos_renyi(3000, 15000, seed=51, n_elabels=3)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
    og = O.Graph.from_edges(G.V, 4, src, dst, lab)
    rng = np.random.default_rng(52)
    qs = _mix(G, rng)
    texts = [q.to_g_text() for q in qs]
    queries = [fm.Query.from_text(t) for t in texts]
    want = []
    for t in texts:
        c, _, _ = O.match(og, O.plan(t, enumerate_aut=0))
        want.append(c)
    yield ctx, g, og, queries, texts, want
    g.close()
    ctx.close()


def test_batch_counts_equal_single_and_oracle(env):
    ctx, g, og, queries, texts, want = env
    single = [fm.match(ctx, g, q, mode=fm.MODE_COUNT).count for q in queries]
    assert single == want
    b = fm.Batch(ctx, g, queries, mode=fm.MODE_COUNT)
    for _ in range(3):                      # first run captures the graph, then replays
        counts, st = b.run()
        assert counts == want
        assert st.batched_queries == len(queries)
    # shared levels: far fewer launches than matching the queries one by one
    assert st.launches < sum(2 * (q.q - 1) for q in queries) // 4
    b.close()


def test_batch_tables_equal_single(env):
    ctx, g, og, queries, texts, want = env
    b = fm.Batch(ctx, g, queries, mode=fm.MODE_TABLE)
    counts, _ = b.run()
    assert counts == want
    for i, q in enumerate(queries):
        rows = b.rows(i, want[i])
        c, single_rows, _ = fm.match_table(ctx, g, q, max_rows=max(1, want[i]))
        assert rows.shape[0] == c == want[i]
        assert np.array_equal(_sorted(rows), _sorted(single_rows))
    b.close()


def test_batch_copy_tables_one_copy(env):
    ctx, g, og, queries, texts, want = env
    b = fm.Batch(ctx, g, queries, mode=fm.MODE_TABLE)
    counts, _ = b.run()
    words_needed = sum(c * q.q for c, q in zip(counts, queries))
    small = np.zeros(max(1, words_needed - 1), dtype=np.uint32)
    with pytest.raises(fm.FMError):
        b.copy_tables(small)
    host = fm.PinnedRows(words_needed + 8, 1)
    words, offs = b.copy_tables(host)
    assert words == words_needed
    flat = host.array
    for i, q in enumerate(queries):
        assert offs[i] is not None
        got = flat[offs[i]: offs[i] + counts[i] * q.q].reshape(-1, q.q)
        assert np.array_equal(got, b.rows(i, counts[i]))
    b.close()


def test_batch_each_query_alone_and_in_the_mix(env):
    ctx, g, og, queries, texts, want = env
    for i in (0, 5, 11, len(queries) - 1):
        alone = fm.Batch(ctx, g, [queries[i]], mode=fm.MODE_COUNT)
        assert alone.run()[0] == [want[i]]
        alone.close()


def test_batch_level_deferral():
    """A tiny SOLN_PREALLOC makes shared levels fill: the persistent engine
    drains them on the device, the level-launch engine on the host; counts
    must not change."""
    G = S.rmat(12, 30000, seed=21, n_elabels=2)
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, 3, src, dst, lab)
    small = fm.Context(prealloc_bytes=256 << 20, soln_prealloc_bytes=8 << 20, output_prealloc_bytes=64 << 20,
                       bank_rows=32)
    g = fm.Graph.from_edges(small, G.V, 3, src, dst, lab)
    qs = [S.query_path(5, [1, 2, 1, 2]), S.query_cycle(4, [1, 1, 2, 2]), S.query_path(4, [2, 2, 1])]
    want = [O.match(og, O.plan(q.to_g_text(), enumerate_aut=0), count_rule=True)[0] for q in qs]
    for engine in (fm.ENGINE_PERSISTENT, fm.ENGINE_LEVELS):
        b = fm.Batch(small, g, [fm.Query.from_text(q.to_g_text()) for q in qs], mode=fm.MODE_COUNT)
        b.set_engine(engine)
        counts, st = b.run()
        assert counts == want
        if engine == fm.ENGINE_LEVELS:
            assert st.launches > 2 * 4     # the host relaunched levels to drain them
        else:
            assert st.launches == 2        # the device drained them inside one launch
        b.close()
    small.close()


def test_batch_tuning_keeps_results(env):
    ctx, g, og, queries, texts, want = env
    b = fm.Batch(ctx, g, queries, mode=fm.MODE_COUNT)
    best = b.tune()
    assert best.wall_ms > 0
    assert b.run()[0] == want
    b.close()


def test_batch_fallback_duplicates_and_single_vertex(env):
    ctx = env[0]
    V = 40
    rng = np.random.default_rng(3)
    s = rng.integers(0, V, 300).astype(np.uint32)
    d = rng.integers(0, V, 300).astype(np.uint32)
    keep = s != d
    s, d = s[keep], d[keep]
    lab = rng.integers(1, 3, len(s)).astype(np.uint32)
    S2, D2, L2 = np.concatenate([s, d, s[:30]]), np.concatenate([d, s, d[:30]]), np.concatenate([lab, lab, lab[:30]])
    g = fm.Graph.from_edges(ctx, V, 3, S2, D2, L2)
    texts = [S.query_cycle(3, [1, 1, 2]).to_g_text(), S.query_path(3, [1, 2]).to_g_text(),
             b"t # 0\n1 0 1 1\nv 0 1\nt # -1"]
    qs = [fm.Query.from_text(t) for t in texts]
    b = fm.Batch(ctx, g, qs, mode=fm.MODE_COUNT)
    counts, st = b.run()
    assert st.single_queries == 3
    assert counts == [fm.match(ctx, g, q, mode=fm.MODE_COUNT).count for q in qs]
    b.close()


def test_batch_with_list_bitmaps(monkeypatch):
    """The batch kernels answer membership from list bitmaps too (lists down
    to 4 entries get one here); counts equal the oracle's."""
    monkeypatch.setenv("FM_BITMAP_MIN_LEN", "4")
    ctx = fm.Context(prealloc_bytes=3 << 30, soln_prealloc_bytes=1 << 30, output_prealloc_bytes=1 << 30,
                     bank_rows=1024)
    G = S.rmat(12, 30000, seed=91, n_elabels=3)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
    assert g.info().bitmaps > 0
    og = O.Graph.from_edges(G.V, 4, src, dst, lab)
    rng = np.random.default_rng(92)
    qs, want = [], []
    while len(qs) < 16:
        k = int(rng.integers(3, 7))
        q = S.query_random_walk(G, k, rng, bias=1.0)
        if q is None:
            continue
        try:
            c = O.match(og, O.plan(q.to_g_text(), enumerate_aut=0), limit=1 << 22, scan_limit=1 << 26)[0]
        except O.OracleError:
            continue
        qs.append(fm.Query.from_text(q.to_g_text()))
        want.append(c)
    b = fm.Batch(ctx, g, qs, mode=fm.MODE_COUNT)
    assert b.run()[0] == want
    b.close()
    g.close()
    ctx.close()


def test_batch_solo_queries_keep_counts_and_tables(env):
    """Queries matched alone inside a run (the single-query engine, table into
    the query's own region) give the same counts and tables as the shared
    launches, in count and table mode, on captured runs and replays, with
    every query alone, some, and back to none; the tuner's choice (read back
    with solo()) keeps them too."""
    ctx, g, og, queries, texts, want = env
    tabled = [i for i, w in enumerate(want) if w <= 1 << 18]
    singles = {i: fm.match_table(ctx, g, queries[i], max_rows=max(1, want[i]))[1] for i in tabled}
    for mode in (fm.MODE_COUNT, fm.MODE_TABLE):
        b = fm.Batch(ctx, g, queries, mode=mode)
        if mode == fm.MODE_TABLE:
            for i in range(len(queries)):
                if i not in tabled:
                    b.set_query_mode(i, fm.MODE_COUNT)
        for pick in (list(range(len(queries))), [0, 3, 6, 7, 11], []):
            for i in range(len(queries)):
                b.set_solo(i, i in pick)
            assert b.solo() == pick
            for _ in range(2):
                counts, st = b.run()
                assert counts == want and st.solo_queries == len(pick)
            if mode == fm.MODE_TABLE:
                for i in tabled:
                    assert np.array_equal(_sorted(b.rows(i, max(1, want[i]))), _sorted(singles[i])), (pick, i)
        best = b.tune()
        assert best.solo_queries == len(b.solo())
        assert b.run()[0] == want
        b.close()
