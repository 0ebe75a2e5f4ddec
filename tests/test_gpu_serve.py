"""Serving (fm_server_*): every request's result is the same alone, in a mix
of concurrent requests, batched with others and under a pool that admits
only a few leases at a time; table requests return the plain tables; a lease
that is too small is retried, never truncated."""
import time

import numpy as np
import pytest

import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MB = 1 << 20


def _sorted(a):
    a = np.asarray(a, dtype=np.uint32)
    return a[np.lexsort(a.T[::-1])] if a.size else a


def _queries(G, og, rng, n=40, cap=1 << 20):
    fixed = [S.query_path(2, [1]), S.query_path(4, [1, 2, 3]), S.query_cycle(3, [1, 2, 3]), S.query_cycle(4, [1, 2, 1, 2]),
             S.query_star(4, [1, 2, 3]), S.query_clique(4, [1, 2, 3]), S.query_path(1, [])]
    out = []
    for q in fixed:
        t = q.to_g_text() if q.k > 1 else b"t # 0\n1 0 1 1\nv 0 1\nt # -1"
        out.append(t)
    while len(out) < n:
        k = int(rng.integers(3, 9))
        q = S.query_random_walk(G, k, rng, tree=bool(len(out) % 4 == 0), bias=1.0)
        if q is None:
            continue
        t = q.to_g_text()
        try:
            c, _, _ = O.match(og, O.plan(t, enumerate_aut=0), limit=1 << 22, scan_limit=1 << 26)
        except O.OracleError:
            continue
        if c <= cap:
            out.append(t)
    return out


@pytest.fixture(scope="module")
def env():
    from forkmatch_gb300 import build
    build.build()
    G = S.rmat(13, 40000, seed=31, n_elabels=8)
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, 9, src, dst, lab)
    texts = _queries(G, og, np.random.default_rng(32))
    ctx = fm.Context(prealloc_bytes=6 << 30, soln_prealloc_bytes=2 << 30, output_prealloc_bytes=2 << 30,
                     bank_rows=1024)
    g = fm.Graph.from_edges(ctx, G.V, 9, src, dst, lab)
    queries = [fm.Query.from_text(t) for t in texts]
    # plain runs (before any server exists) and the oracle
    want = [fm.match(ctx, g, q, mode=fm.MODE_COUNT).count for q in queries]
    oracle = [O.match(og, O.plan(t, enumerate_aut=0))[0] if fm.Query.from_text(t).q > 1 else G.V for t in texts]
    assert want == oracle
    tables = [_sorted(fm.match_table(ctx, g, q, max_rows=max(1, c))[1]) for q, c in zip(queries, want)]
    yield dict(G=G, src=src, dst=dst, lab=lab, ctx=ctx, g=g, queries=queries, texts=texts, want=want, tables=tables)
    g.close()
    ctx.close()


def _run_all(srv, queries, mode=fm.MODE_COUNT, rows=None):
    tickets = [srv.submit(q, mode=mode, host_rows=None if rows is None else rows[i]) for i, q in enumerate(queries)]
    res = [srv.poll(t) for t in tickets]
    for t in tickets:
        srv.release(t)
    return res


def test_each_result_alone_and_in_the_mix(env):
    srv = fm.Server(env["ctx"], env["g"], slots=4, max_batch=8)
    try:
        alone = []
        for q in env["queries"]:
            t = srv.submit(q)
            r = srv.poll(t)
            assert r.done and r.status == fm.FM_OK
            alone.append(r.count)
            srv.release(t)
        assert alone == env["want"]
        for _ in range(3):
            res = _run_all(srv, env["queries"])
            assert [r.status for r in res] == [fm.FM_OK] * len(res)
            assert [r.count for r in res] == env["want"]
        st = srv.stats()
        assert st.completed == st.submitted == 4 * len(env["queries"])
        assert st.queued == 0 and st.running == 0
        assert st.pool_free == st.pool_bytes
    finally:
        srv.close()


def test_batching_shares_launches_without_changing_counts(env):
    srv = fm.Server(env["ctx"], env["g"], slots=1, max_batch=64)
    try:
        qs = env["queries"] * 3
        res = _run_all(srv, qs)
        assert [r.count for r in res] == env["want"] * 3
        assert max(r.batch for r in res) > 1
        assert srv.stats().batches >= 1
    finally:
        srv.close()


def test_table_requests_return_the_plain_tables(env):
    srv = fm.Server(env["ctx"], env["g"], slots=3)
    try:
        rows = [np.zeros(max(1, c) * q.q, dtype=np.uint32) for q, c in zip(env["queries"], env["want"])]
        res = _run_all(srv, env["queries"], mode=fm.MODE_TABLE, rows=rows)
        for i, (r, q) in enumerate(zip(res, env["queries"])):
            assert r.status == fm.FM_OK and r.count == env["want"][i] and r.rows_copied == r.count
            got = _sorted(rows[i][: r.count * q.q].reshape(-1, q.q))
            assert np.array_equal(got, env["tables"][i])
    finally:
        srv.close()


def test_small_leases_retry_instead_of_truncating(env):
    """max_lease caps the first table lease below the largest tables: those
    requests run again with an exact lease and still return every row."""
    big = int(np.argmax([c * q.q for c, q in zip(env["want"], env["queries"])]))
    q = env["queries"][big]
    c = env["want"][big]
    assert c * q.q * 4 > 2 * MB
    srv = fm.Server(env["ctx"], env["g"], slots=2, min_lease_bytes=2 * MB, max_lease_bytes=2 * MB)
    try:
        buf = np.zeros(c * q.q, dtype=np.uint32)
        t = srv.submit(q, mode=fm.MODE_TABLE, host_rows=buf)
        r = srv.poll(t)
        assert r.status == fm.FM_OK and r.count == c and r.rows_copied == c and r.attempts == 2
        assert np.array_equal(_sorted(buf.reshape(-1, q.q)), env["tables"][big])
        srv.release(t)
        # a caller buffer smaller than the table: exact count, truncated rows
        small = np.zeros((c // 2) * q.q, dtype=np.uint32)
        t = srv.submit(q, mode=fm.MODE_TABLE, host_rows=small)
        r = srv.poll(t)
        assert r.status == fm.FM_ERR_OUTPUT_OVERFLOW and r.truncated and r.count == c and r.rows_copied == c // 2
        srv.release(t)
    finally:
        srv.close()


def test_pool_admits_only_what_fits(env):
    """A pool of a few hundred MiB and fixed 96 MiB leases: at most a few
    requests hold leases at once although 8 slots are idle; all counts exact."""
    G = env["G"]
    ctx = fm.Context(prealloc_bytes=8 * 64 * MB + 400 * MB, soln_prealloc_bytes=64 * MB, output_prealloc_bytes=64 * MB,
                     bank_rows=1024)
    g = fm.Graph.from_edges(ctx, G.V, 9, env["src"], env["dst"], env["lab"])
    srv = fm.Server(ctx, g, slots=8, min_lease_bytes=96 * MB, max_lease_bytes=96 * MB)
    try:
        st0 = srv.stats()
        fit = st0.pool_bytes // (96 * MB)
        assert 2 <= fit < 8
        # every request here leases exactly 96 MiB (q >= 3: level buffers)
        pick = [i for i, q in enumerate(env["queries"]) if q.q >= 3]
        tickets = [srv.submit(env["queries"][i]) for i in pick * 2]
        peak_running = 0
        while srv.stats().completed < len(tickets):
            peak_running = max(peak_running, srv.stats().running)
            time.sleep(0.0005)
        res = [srv.poll(t) for t in tickets]
        assert [r.count for r in res] == [env["want"][i] for i in pick] * 2
        st = srv.stats()
        assert st.pool_peak_used <= st.pool_bytes
        assert peak_running <= fit
        assert max(r.queue_ms for r in res) > 0
    finally:
        srv.close()
        g.close()
        ctx.close()


def test_request_work_limit(env):
    big = int(np.argmax(env["want"]))
    q, c = env["queries"][big], env["want"][big]
    assert c > 1000
    srv = fm.Server(env["ctx"], env["g"], slots=2, max_batch=8, work_limit=1000)
    try:
        t = srv.submit(q)
        r = srv.poll(t)
        assert r.status == fm.FM_ERR_LIMIT and r.batch == 1 and r.error
        srv.release(t)
    finally:
        srv.close()
    # a limit no request reaches: exact counts, and no batching under a limit
    srv = fm.Server(env["ctx"], env["g"], slots=2, max_batch=8, work_limit=1 << 40)
    try:
        res = _run_all(srv, env["queries"])
        assert [r.count for r in res] == env["want"]
        assert max(r.batch for r in res) == 1
    finally:
        srv.close()


def test_server_owns_the_slab(env):
    ctx, g, q = env["ctx"], env["g"], env["queries"][3]
    srv = fm.Server(ctx, g, slots=1)
    try:
        with pytest.raises(fm.FMError):
            fm.match(ctx, g, q, mode=fm.MODE_COUNT)
        with pytest.raises(fm.FMError):
            fm.Batch(ctx, g, [q])
        with pytest.raises(fm.FMError):
            fm.Server(ctx, g)
    finally:
        srv.close()
    assert fm.match(ctx, g, q, mode=fm.MODE_COUNT).count == env["want"][3]
