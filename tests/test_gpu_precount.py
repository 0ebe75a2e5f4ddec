"""Pre-count (count mode, last depth with one back edge): depth q-2 counts each
survivor's extensions -- the length of that one list minus the row's vertices
found in it -- instead of storing the survivor for a last level launch.

Counts must equal the oracle's enumeration, the per-level work counters must
equal the oracle's as if the last depth had been launched, and the results
must equal the library's own with the last depth launched (FM_PRE_COUNT=0, read
once per process, so that side runs in a child process).  Lists of every kind
are exercised: inline (<= 3 entries), binary-searched in lockstep (no
bitmaps), and bitmaps down to 4 entries.  Integer work: no tolerance."""
import json
import math
import os
import subprocess
import sys

import numpy as np
import pytest

import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S
from oracle import oracle as O
from tests.helpers import complete_graph

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ctx():
    from forkmatch_gb300 import build
    build.build()
    c = fm.Context(prealloc_bytes=2 << 30, soln_prealloc_bytes=512 << 20, output_prealloc_bytes=256 << 20,
                   bank_rows=256)
    yield c
    c.close()


def _queries(G, seed):
    """Paths (the new vertex is the last back edge's ancestor), stars (the
    ancestor is the centre, matched long before), random walk trees and
    cycles (two back edges: never pre-counted), 3 to 6 vertices."""
    rng = np.random.default_rng(seed)
    L = G.n_elabels
    qs = [S.query_path(3, [1, 2]), S.query_path(4, [1, 1, 2]), S.query_path(5, [2, 1, 2, 1]),
          S.query_path(6, [1, 2, 3 % L + 1, 1, 2]), S.query_star(4, [1, 2, 2]), S.query_star(5, [1, 1, 2, 2]),
          S.query_cycle(4, [1, 2, 1, 2])]
    for i in range(24):
        q = S.query_random_walk(G, int(rng.integers(3, 7)), rng, tree=i % 2 == 0, bias=1.0)
        if q is not None:
            qs.append(q)
    return [q.to_g_text() for q in qs]


def _oracle(og, text, limit=1 << 27):
    p = O.plan(text, enumerate_aut=0)
    try:
        c, _, st = O.match(og, p, limit=limit)
    except O.OracleError:
        return None
    return p, c, st


@pytest.mark.parametrize("bitmaps", ["default", "none", "short"])
def test_pre_count_equals_enumeration_and_work_counters(ctx, monkeypatch, bitmaps):
    if bitmaps == "none":
        monkeypatch.setenv("FM_BITMAP_BYTES", "0")
    if bitmaps == "short":
        monkeypatch.setenv("FM_BITMAP_MIN_LEN", "4")
    G = S.rmat(12, 20000, seed=43, n_elabels=3)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
    og = O.Graph.from_edges(G.V, 4, src, dst, lab)
    assert (g.info().bitmaps == 0) == (bitmaps == "none")
    pre = done = 0
    for text in _queries(G, 7):
        o = _oracle(og, text)
        if o is None:
            continue
        p, oc, ost = o
        q = fm.Query.from_text(text)
        assert fm.match(ctx, g, q, mode=fm.MODE_COUNT).count == oc
        pre += p.q >= 3 and p.nreq[p.q - 1] == 1
        for engine in (fm.ENGINE_LEVELS, fm.ENGINE_PERSISTENT):
            r = fm.match(ctx, g, q, mode=fm.MODE_COUNT, order=fm.ORDER_REFERENCE, engine=engine)
            assert r.count == oc
            assert r.pre_counted == (1 if p.q >= 3 and p.nreq[p.q - 1] == 1 else 0)
            for d in range(2, p.q):
                assert r.level[d].lookups == ost.lookups[d], ("lookups", d, engine)
                assert r.level[d].list_words == ost.list_words[d], ("list_words", d, engine)
                assert r.level[d].parents == ost.partials[d - 1], ("parents", d, engine)
            for d in range(1, p.q - 1):
                assert r.level[d].produced == ost.partials[d], ("produced", d, engine)
        done += 1
    assert done >= 12 and pre >= 10
    g.close()


def test_pre_count_in_batches(ctx):
    """Count batches and count-only queries inside a table batch, both
    engines: each count equals the single-query count."""
    G = S.rmat(12, 20000, seed=44, n_elabels=3)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
    og = O.Graph.from_edges(G.V, 4, src, dst, lab)
    texts = [t for t in _queries(G, 8) if _oracle(og, t) is not None]     # bounded work
    queries = [fm.Query.from_text(t) for t in texts]
    want = [fm.match(ctx, g, q, mode=fm.MODE_COUNT).count for q in queries]
    small = [i for i, w in enumerate(want) if w <= 1 << 16]
    for engine in (fm.ENGINE_LEVELS, fm.ENGINE_PERSISTENT):
        b = fm.Batch(ctx, g, queries, mode=fm.MODE_COUNT)
        b.set_engine(engine)
        for _ in range(2):
            assert b.run()[0] == want
        b.close()
        b = fm.Batch(ctx, g, queries, mode=fm.MODE_TABLE)
        b.set_engine(engine)
        for i in range(len(queries)):
            if i not in small:
                b.set_query_mode(i, fm.MODE_COUNT)
        for _ in range(2):
            assert b.run()[0] == want
        for i in small[:4]:
            _, rows, _ = fm.match_table(ctx, g, queries[i], max_rows=max(1, want[i]))
            br = b.rows(i, max(1, want[i]))
            assert np.array_equal(rows[np.lexsort(rows.T[::-1])], br[np.lexsort(br.T[::-1])])
        b.close()
    g.close()


def test_pre_count_with_self_loops_and_complete_graphs(ctx):
    """K_n plus a self-loop on every vertex: a vertex is in its own list, and
    the count must still exclude it (injectivity): n!/(n-k)! paths and
    stars of k vertices."""
    n = 9
    V, s, d, l = complete_graph(n)
    loops = np.arange(n, dtype=np.uint32)
    s, d = np.concatenate([s, loops]), np.concatenate([d, loops])
    l = np.ones(len(s), dtype=np.uint32)
    g = fm.Graph.from_edges(ctx, V, 2, s, d, l)
    for k in (3, 4, 5, 6):
        for text in (S.query_path(k, [1] * (k - 1)).to_g_text(), S.query_star(k, [1] * (k - 1)).to_g_text()):
            r = fm.match(ctx, g, fm.Query.from_text(text), mode=fm.MODE_COUNT)
            assert r.pre_counted == 1 and r.count == math.perm(n, k)
    g.close()


_LAUNCHED = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S
texts = [t.encode() for t in json.loads(sys.argv[2])]
G = S.rmat(12, 20000, seed=43, n_elabels=3)
src, dst, lab = G.directed()
ctx = fm.Context(prealloc_bytes=2 << 30, soln_prealloc_bytes=512 << 20, output_prealloc_bytes=256 << 20,
                 bank_rows=256)
g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
out = []
for t in texts:
    r = fm.match(ctx, g, fm.Query.from_text(t), mode=fm.MODE_COUNT, order=fm.ORDER_REFERENCE)
    out.append([r.count, r.pre_counted] + [[r.level[d].parents, r.level[d].lookups, r.level[d].list_words,
                                            r.level[d].produced] for d in range(1, r.q)])
print("LAUNCHED " + json.dumps(out))
"""


def test_pre_count_equals_the_launched_last_depth(ctx):
    G = S.rmat(12, 20000, seed=43, n_elabels=3)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
    og = O.Graph.from_edges(G.V, 4, src, dst, lab)
    texts = [t for t in _queries(G, 9) if _oracle(og, t) is not None]     # bounded work
    env = dict(os.environ, FM_PRE_COUNT="0")
    r = subprocess.run([sys.executable, "-c", _LAUNCHED, ROOT, json.dumps([t.decode() for t in texts])], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    launched = json.loads(r.stdout.split("LAUNCHED ", 1)[1])
    n_pre = 0
    for t, other in zip(texts, launched):
        res = fm.match(ctx, g, fm.Query.from_text(t), mode=fm.MODE_COUNT, order=fm.ORDER_REFERENCE)
        assert other[1] == 0
        n_pre += res.pre_counted
        mine = [res.count, 0] + [[res.level[d].parents, res.level[d].lookups, res.level[d].list_words,
                                  res.level[d].produced] for d in range(1, res.q)]
        # the last depth's "produced" is its count in both runs
        assert mine == other, t
    assert n_pre >= 8
    g.close()
