"""The persistent engine (one cooperative launch per match or batch, level
passes scheduled on the device from per-depth work queues) against the level
launch engine and the oracle: identical counts, tables and per-level work
counters, with level buffers from ample down to a few chunks (so that the
device drains levels depth first many times), and a grid-wide wait that runs
out ends the match with FM_ERR_DEVICE while the context stays usable."""
import numpy as np
import pytest

import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sorted(a):
    a = np.asarray(a, dtype=np.uint32)
    return a[np.lexsort(a.T[::-1])] if a.size else a


@pytest.fixture(scope="module")
def graph():
    from forkmatch_gb300 import build
    build.build()
    G = S.rmat(12, 30000, seed=21, n_elabels=2)
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, 3, src, dst, lab)
    rng = np.random.default_rng(5)
    cands = [S.query_path(4, [1, 2, 1]), S.query_cycle(4, [1, 2, 1, 2]), S.query_star(4, [1, 1, 2]),
             S.query_clique(4, [1, 2]), S.query_path(2, [1])]
    for _ in range(40):
        q = S.query_random_walk(G, int(rng.integers(4, 7)), rng, min_density=0.5, bias=1.0)
        if q is not None:
            cands.append(q)
    # the oracle's counts (count rule: exact, pinned against enumeration on
    # the CPU); queries it cannot finish within its node limit are dropped
    texts, want = [], []
    for q in cands:
        t = q.to_g_text()
        try:
            c = O.match(og, O.plan(t, enumerate_aut=0), count_rule=True, limit=1 << 25)[0]
        except O.OracleError:
            continue
        if c > 500_000_000:          # keeps the level-launch engine's host drains short
            continue
        texts.append(t)
        want.append(c)
        if len(texts) == 9:
            break
    assert len(texts) >= 7
    return G, (src, dst, lab), og, texts, want


@pytest.mark.parametrize("soln_mib", [1024, 64, 24])
def test_engines_agree_from_ample_to_tiny_level_buffers(graph, soln_mib):
    G, (src, dst, lab), og, texts, want = graph
    ctx = fm.Context(prealloc_bytes=(soln_mib << 20) + (256 << 20), soln_prealloc_bytes=soln_mib << 20,
                     output_prealloc_bytes=128 << 20, bank_rows=32)
    g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
    deferred = 0
    for t, w in zip(texts, want):
        q = fm.Query.from_text(t)
        a = fm.match(ctx, g, q, mode=fm.MODE_COUNT, engine=fm.ENGINE_PERSISTENT)
        b = fm.match(ctx, g, q, mode=fm.MODE_COUNT, engine=fm.ENGINE_LEVELS)
        assert a.count == b.count == w
        assert a.engine == fm.ENGINE_PERSISTENT and a.launches == 1
        for d in range(1, q.q):
            la, lb = a.level[d], b.level[d]
            assert (la.parents, la.lookups, la.list_words) == (lb.parents, lb.lookups, lb.list_words), d
            if d + 1 < q.q:
                assert la.produced == lb.produced, d
        deferred += a.passes > q.q - 1 - a.pre_counted   # more passes than launched depths
        if w <= 1 << 20:
            ca, ra, _ = fm.match_table(ctx, g, q, max_rows=max(1, w))
            assert ca == w
            buf = np.zeros(max(1, w) * q.q, dtype=np.uint32)
            rb = fm.match(ctx, g, q, mode=fm.MODE_TABLE, host_rows=buf, engine=fm.ENGINE_LEVELS)
            assert np.array_equal(_sorted(ra), _sorted(buf[: rb.rows_copied * q.q].reshape(-1, q.q)))
    if soln_mib <= 64:
        assert deferred >= 1          # the device drained at least one level depth first
    g.close()
    ctx.close()


def test_persistent_wait_that_runs_out_returns_an_error_and_the_context_survives(graph):
    """One block never arrives at the first grid barrier (a flag nothing
    sets): every other block's wait runs out after wait_limit_ms, the kernel
    returns, fm_match reports FM_ERR_DEVICE, and the next match on the same
    context is exact."""
    G, (src, dst, lab), og, texts, want = graph
    ctx = fm.Context(prealloc_bytes=1 << 30, soln_prealloc_bytes=256 << 20, output_prealloc_bytes=128 << 20,
                     bank_rows=32)
    g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
    q = fm.Query.from_text(texts[0])
    r = fm.match(ctx, g, q, mode=fm.MODE_COUNT, engine=fm.ENGINE_PERSISTENT, wait_limit_ms=200,
                 test_stall_barrier=True, allow_device_error=True)
    assert r.status == fm.FM_ERR_DEVICE and r.engine == fm.ENGINE_PERSISTENT
    assert b"wait" in fm.lib().fm_last_error()
    assert r.max_wait_ns >= 150_000_000
    for t, w in zip(texts, want):
        assert fm.match(ctx, g, fm.Query.from_text(t), mode=fm.MODE_COUNT).count == w
    g.close()
    ctx.close()


def test_batch_engines_agree(graph):
    G, (src, dst, lab), og, texts, want = graph
    ctx = fm.Context(prealloc_bytes=1 << 30, soln_prealloc_bytes=48 << 20, output_prealloc_bytes=512 << 20,
                     bank_rows=32)
    g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
    queries = [fm.Query.from_text(t) for t in texts]
    tabled = [i for i, w in enumerate(want) if w <= 1 << 20]     # the others are counted only
    for mode in (fm.MODE_COUNT, fm.MODE_TABLE):
        got = {}
        for engine in (fm.ENGINE_PERSISTENT, fm.ENGINE_LEVELS):
            b = fm.Batch(ctx, g, queries, mode=mode)
            b.set_engine(engine)
            if mode == fm.MODE_TABLE:
                for i in range(len(queries)):
                    if i not in tabled:
                        b.set_query_mode(i, fm.MODE_COUNT)
            for _ in range(2):                 # first run captures, the second replays
                counts, st = b.run()
                assert counts == want
                assert st.persistent == (engine == fm.ENGINE_PERSISTENT)
            if mode == fm.MODE_TABLE:
                got[engine] = [_sorted(b.rows(i, max(1, want[i]))) for i in tabled]
            b.close()
        if mode == fm.MODE_TABLE:
            for x, y in zip(got[fm.ENGINE_PERSISTENT], got[fm.ENGINE_LEVELS]):
                assert np.array_equal(x, y)
    g.close()
    ctx.close()


_STAGED_CHECK = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S
from oracle import oracle as O
G = S.rmat(12, 40000, seed=23, n_elabels=2)
src, dst, lab = G.directed()
og = O.Graph.from_edges(G.V, 3, src, dst, lab)
ctx = fm.Context(prealloc_bytes=1 << 30, soln_prealloc_bytes=64 << 20, output_prealloc_bytes=256 << 20, bank_rows=32)
g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
qs = [S.query_cycle(4, [1, 2, 1, 2]), S.query_clique(4, [1, 2]), S.query_clique(5, [2, 1]),
      S.query_cycle(4, [1, 1, 2, 2])]
want = [O.match(og, O.plan(q.to_g_text(), enumerate_aut=0))[0] for q in qs]
queries = [fm.Query.from_text(q.to_g_text()) for q in qs]
for engine in (fm.ENGINE_PERSISTENT, fm.ENGINE_LEVELS):
    got = [fm.match(ctx, g, q, mode=fm.MODE_COUNT, engine=engine).count for q in queries]
    assert got == want, (engine, got, want)
for qq, q, w in zip(qs, queries, want):
    if w <= 1 << 20:
        c, rows, _ = fm.match_table(ctx, g, q, max_rows=max(1, w))
        o = O.match(og, O.plan(qq.to_g_text(), enumerate_aut=0), table=True, table_cap=max(1, w))[1]
        a = rows[np.lexsort(rows.T[::-1])]
        b = o[np.lexsort(o.T[::-1])]
        assert c == w and np.array_equal(a, b)
b = fm.Batch(ctx, g, queries, mode=fm.MODE_COUNT)
for _ in range(2):
    counts, _ = b.run()
    assert counts == want, (counts, want)
print("staged ok", want)
"""


@pytest.mark.parametrize("words", [64, 1024])
def test_staged_membership_lists_give_identical_results(words):
    """With the per-warp stage on (FM_STAGE_WORDS, read once per process, so
    the check runs in a child process), membership lists copied into shared
    memory by TMA bulk copies give the oracle's counts and tables in both
    engines and in a batch; 64 words forces most lists to stay in global
    memory beside the staged ones."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FM_STAGE_WORDS=str(words))
    r = subprocess.run([sys.executable, "-c", _STAGED_CHECK, root], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "staged ok" in r.stdout


def test_count_only_queries_in_a_table_batch(graph):
    """Queries set to count only in a table-mode batch keep exact counts (the
    count rule on their last level), get no table region and raise no
    truncation; the other queries' tables are unchanged."""
    G, (src, dst, lab), og, texts, want = graph
    ctx = fm.Context(prealloc_bytes=2 << 30, soln_prealloc_bytes=256 << 20, output_prealloc_bytes=1 << 30,
                     bank_rows=32)
    g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
    queries = [fm.Query.from_text(t) for t in texts]
    counted = [w > 1 << 20 for w in want]        # tables too large to keep
    assert any(counted) and not all(counted)
    for engine in (fm.ENGINE_PERSISTENT, fm.ENGINE_LEVELS):
        b = fm.Batch(ctx, g, queries, mode=fm.MODE_TABLE)
        b.set_engine(engine)
        for i, c in enumerate(counted):
            if c:
                b.set_query_mode(i, fm.MODE_COUNT)
        for _ in range(2):
            counts, _ = b.run()
            assert counts == want
        for i, (q, w) in enumerate(zip(queries, want)):
            rows = b.rows(i, max(1, w) if not counted[i] else 1)
            if counted[i]:
                assert rows.shape[0] == 0
            else:
                c, single, _ = fm.match_table(ctx, g, q, max_rows=max(1, w))
                assert rows.shape[0] == w and np.array_equal(_sorted(rows), _sorted(single))
        b.close()
    g.close()
    ctx.close()
