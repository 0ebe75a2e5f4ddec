"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Every test here runs the product kernels on the GPU and compares with the
oracle (counts bit-exact, tables as sorted row sets, per-level work counters
exact) or with closed-form counts.  Integer work: no tolerance anywhere."""
import math
import os

import numpy as np
import pytest

import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S
from oracle import oracle as O
from tests.helpers import (complete_graph, cycle_graph, golden_graphs, make_graph, reference_matches, star_graph,
                           table_sha)

pytestmark = pytest.mark.gpu

GB = 1 << 30


@pytest.fixture(scope="module")
def ctx():
    from forkmatch_gb300 import build
    build.build()
    c = fm.Context(prealloc_bytes=3 * GB, soln_prealloc_bytes=1 * GB, output_prealloc_bytes=1 * GB,
                   bank_rows=1024)
    yield c
    c.close()


def sorted_rows(a):
    a = np.asarray(a, dtype=np.uint32)
    if a.size == 0:
        return a.reshape(0, 0)
    idx = np.lexsort(a.T[::-1])
    return a[idx]


def check_case(ctx, g, og, qtext, expect_count=None, table=True, max_rows=1 << 20):
    p = O.plan(qtext, enumerate_aut=0)
    oc, orows, ost = O.match(og, p, table=table, table_cap=max_rows)
    if expect_count is not None:
        assert oc == expect_count
    q = fm.Query.from_text(qtext)
    # the cost-based order must not change the result
    assert fm.match(ctx, g, q, mode=fm.MODE_COUNT, order=fm.ORDER_AUTO).count == oc
    # with the reference order the per-level work equals the oracle's exactly
    r = fm.match(ctx, g, q, mode=fm.MODE_COUNT, order=fm.ORDER_REFERENCE)
    assert r.count == oc
    # depth 1: the roots are the vertices with an e-line of one depth-1 label
    # (every other vertex fails the reference's root lookup, src/smsm.cu:835)
    if r.launches == 0:
        # a query label is absent from the graph: no launch is needed
        assert oc == 0
        return oc
    if p.q > 1:
        with_label = [og.sources(p.req_label[1][i]) for i in range(p.nreq[1])]
        assert r.level[1].parents == min(with_label)
        assert r.level[1].lookups == min(with_label) * p.nreq[1]
    for d in range(2, p.q):
        assert r.level[d].lookups == ost.lookups[d], ("lookups", d)
        assert r.level[d].list_words == ost.list_words[d], ("list_words", d)
        assert r.level[d].parents == ost.partials[d - 1], ("parents", d)
    for d in range(1, p.q - 1):
        assert r.level[d].produced == ost.partials[d], ("produced", d)
    if table and oc <= max_rows:
        want = sorted_rows(orows)
        for order in (fm.ORDER_AUTO, fm.ORDER_REFERENCE):
            cnt, rows, r2 = fm.match_table(ctx, g, q, max_rows=max_rows, order=order)
            assert cnt == oc
            assert np.array_equal(sorted_rows(rows), want)
    return oc


def test_golden_cases_count_table_and_work_counters(ctx):
    n = 0
    for case, G, text in golden_graphs():
        g = fm.Graph.from_text(ctx, text)
        og = O.Graph.parse(text)
        info = g.info()
        assert info.edges == case["E"] and info.vertices == case["V"]
        for e in case["cases"]:
            c = check_case(ctx, g, og, e["text"].encode(), expect_count=e["count"])
            n += 1
            assert c == e["count"]
    assert n > 50


def test_counts_and_tables_equal_the_reference_gpu_build(ctx):
    """Every query the reference's own GPU matcher ran (tests/golden/
    ref_matches.json): our count and sorted table equal its count and table,
    under both engines, except for the cases the reference gets wrong (edge
    label 1 on a graph whose label count makes it write past its label-graph
    table), where they equal the oracle's."""
    graphs = {}
    n = 0
    for g, case, ref in reference_matches():
        key = g["graph"]
        if key not in graphs:
            graphs[key] = fm.Graph.from_text(ctx, make_graph(g["params"]).to_g_text())
        q = fm.Query.from_text(case["text"].encode())
        want_count = ref["count"] if ref["agrees_with_oracle"] else ref["oracle_count"]
        want_sha = ref["table_sha256"] if ref["agrees_with_oracle"] else ref["oracle_table_sha256"]
        for engine in (fm.ENGINE_PERSISTENT, fm.ENGINE_LEVELS):
            assert fm.match(ctx, graphs[key], q, mode=fm.MODE_COUNT, engine=engine).count == want_count
        cnt, rows, _ = fm.match_table(ctx, graphs[key], q, max_rows=max(1, want_count))
        assert cnt == want_count and table_sha(rows) == want_sha
        n += 1
    assert n >= 60
    for g in graphs.values():
        g.close()


@pytest.mark.parametrize("n", [5, 9, 33])
def test_complete_graph_closed_forms(ctx, n):
    V, s, d, l = complete_graph(n)
    g = fm.Graph.from_edges(ctx, V, 2, s, d, l)
    for qq, want in [(S.query_cycle(3, [1] * 3), n * (n - 1) * (n - 2)),
                     (S.query_cycle(4, [1] * 4), n * (n - 1) * (n - 2) * (n - 3)),
                     (S.query_clique(4, [1]), math.perm(n, 4)),
                     (S.query_clique(5, [1]), math.perm(n, 5))]:
        r = fm.match(ctx, g, fm.Query.from_text(qq.to_g_text()), mode=fm.MODE_COUNT)
        assert r.count == want


def test_star_and_cycle_closed_forms(ctx):
    V, s, d, l = star_graph(40)
    g = fm.Graph.from_edges(ctx, V, 2, s, d, l)
    for k in (2, 3, 4):
        r = fm.match(ctx, g, fm.Query.from_text(S.query_star(k + 1, [1] * k).to_g_text()), mode=fm.MODE_COUNT)
        assert r.count == math.perm(40, k)
    V, s, d, l = cycle_graph(1000)
    g = fm.Graph.from_edges(ctx, V, 2, s, d, l)
    for k in (2, 5, 9):
        r = fm.match(ctx, g, fm.Query.from_text(S.query_path(k, [1] * k).to_g_text()), mode=fm.MODE_COUNT)
        assert r.count == 2000


def test_heavy_chunks_split_across_warps(ctx):
    """Hub lists longer than one warp's share (> 2048 candidate slots per
    chunk) are cut into pieces for every warp; counts and rows must not change.
    K_{2,n}: 4-cycles = 8 * C(n, 2), 2-stars centred anywhere = 2*n*(n-1) + n*2."""
    n = 3000
    hubs = np.array([0, 1], dtype=np.uint32)
    leaves = np.arange(2, n + 2, dtype=np.uint32)
    a = np.repeat(hubs, n)
    b = np.tile(leaves, 2)
    src = np.concatenate([a, b])
    dst = np.concatenate([b, a])
    lab = np.ones(len(src), dtype=np.uint32)
    g = fm.Graph.from_edges(ctx, n + 2, 2, src, dst, lab)
    og = O.Graph.from_edges(n + 2, 2, src, dst, lab)
    c4 = S.query_cycle(4, [1] * 4).to_g_text()
    want = 8 * math.comb(n, 2)
    for order in (fm.ORDER_AUTO, fm.ORDER_REFERENCE):
        assert fm.match(ctx, g, fm.Query.from_text(c4), mode=fm.MODE_COUNT, order=order).count == want
    cnt, rows, _ = fm.match_table(ctx, g, fm.Query.from_text(c4), max_rows=want)
    assert cnt == want
    ocnt, orows, _ = O.match(og, O.plan(c4, enumerate_aut=0), table=True, table_cap=want)
    assert np.array_equal(sorted_rows(rows), sorted_rows(orows))
    p3 = S.query_path(3, [1, 1]).to_g_text()
    assert fm.match(ctx, g, fm.Query.from_text(p3), mode=fm.MODE_COUNT).count == 2 * n * (n - 1) + n * 2


@pytest.mark.parametrize("min_len,budget", [("4", None), ("16", "4194304"), (None, "0")])
def test_list_bitmaps_give_identical_results(ctx, monkeypatch, min_len, budget):
    """Membership bitmaps for long lists (down to 4 entries, under a small
    budget that covers only the longest, or none at all): counts, tables and
    work counters equal the oracle's."""
    if min_len is not None:
        monkeypatch.setenv("FM_BITMAP_MIN_LEN", min_len)
    if budget is not None:
        monkeypatch.setenv("FM_BITMAP_BYTES", budget)
    G = S.rmat(13, 50000, seed=41, n_elabels=3)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
    og = O.Graph.from_edges(G.V, 4, src, dst, lab)
    info = g.info()
    if budget == "0":
        assert info.bitmaps == 0
    else:
        assert info.bitmaps > 0 and info.bitmap_min_len >= int(min_len)
        assert info.bitmap_bytes <= (int(budget) if budget else 2 << 30)
    rng = np.random.default_rng(42)
    done = 0
    for i in range(40):
        k = int(rng.integers(3, 7))
        q = S.query_random_walk(G, k, rng, tree=bool(i % 3 == 0), bias=1.0)
        if q is None:
            continue
        try:
            O.match(og, O.plan(q.to_g_text(), enumerate_aut=0), limit=1 << 21, scan_limit=1 << 25)
        except O.OracleError:
            continue
        check_case(ctx, g, og, q.to_g_text(), table=True, max_rows=1 << 21)
        done += 1
    assert done >= 8
    g.close()


def test_work_limit_stops_early_with_a_lower_bound(ctx):
    """K_{2,n}: 8 * C(n, 2) four-cycles.  A work limit far below stops the last
    level (count mode and table mode) and the middle levels (host check), and
    reports FM_ERR_LIMIT with a count between the limit and the full count."""
    n = 3000
    a = np.repeat(np.array([0, 1], dtype=np.uint32), n)
    b = np.tile(np.arange(2, n + 2, dtype=np.uint32), 2)
    src, dst = np.concatenate([a, b]), np.concatenate([b, a])
    lab = np.ones(len(src), dtype=np.uint32)
    g = fm.Graph.from_edges(ctx, n + 2, 2, src, dst, lab)
    c4 = fm.Query.from_text(S.query_cycle(4, [1] * 4).to_g_text())
    full = 8 * math.comb(n, 2)
    assert fm.match(ctx, g, c4, mode=fm.MODE_COUNT, work_limit=full + 1).count == full
    for mode in (fm.MODE_COUNT, fm.MODE_TABLE):
        r = fm.match(ctx, g, c4, mode=mode, work_limit=1 << 20, allow_limit=True)
        assert r.status == fm.FM_ERR_LIMIT
        assert (1 << 20) < r.count < full
    with pytest.raises(fm.FMError):
        fm.match(ctx, g, c4, mode=fm.MODE_COUNT, work_limit=1 << 20)
    # partial matches: a 5-path has 2 * n * (n - 1) * ... middle rows
    p5 = fm.Query.from_text(S.query_path(5, [1] * 4).to_g_text())
    r = fm.match(ctx, g, p5, mode=fm.MODE_COUNT, work_limit=1000, allow_limit=True)
    assert r.status == fm.FM_ERR_LIMIT
    g.close()


def test_label_mismatch_and_absent_label(ctx):
    V, s, d, l = complete_graph(6, label=2)
    g = fm.Graph.from_edges(ctx, V, 3, s, d, l)
    assert fm.match(ctx, g, fm.Query.from_text(S.query_cycle(3, [1] * 3).to_g_text())).count == 0
    # label 7 is beyond the graph's label slots: no embedding, no out-of-range lookup
    assert fm.match(ctx, g, fm.Query.from_text(S.query_path(3, [7, 7]).to_g_text())).count == 0


def test_duplicate_edges_min_multiplicity(ctx):
    rng = np.random.default_rng(3)
    V = 40
    m = 400
    src = rng.integers(0, V, m).astype(np.uint32)
    dst = rng.integers(0, V, m).astype(np.uint32)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    lab = rng.integers(1, 3, len(src)).astype(np.uint32)
    # both directions, then duplicate a third of the e-lines
    S2 = np.concatenate([src, dst])
    D2 = np.concatenate([dst, src])
    L2 = np.concatenate([lab, lab])
    dup = rng.random(len(S2)) < 0.33
    S2 = np.concatenate([S2, S2[dup]])
    D2 = np.concatenate([D2, D2[dup]])
    L2 = np.concatenate([L2, L2[dup]])
    g = fm.Graph.from_edges(ctx, V, 3, S2, D2, L2)
    assert g.info().has_duplicates
    og = O.Graph.from_edges(V, 3, S2, D2, L2)
    for qq in [S.query_path(3, [1, 2]), S.query_cycle(3, [1, 1, 2]), S.query_cycle(4, [1, 2, 1, 2]),
               S.query_clique(4, [1, 2]), S.query_star(4, [1, 1, 2])]:
        check_case(ctx, g, og, qq.to_g_text())


def test_rmat_random_walk_queries(ctx):
    G = S.rmat(14, 60000, seed=11, n_elabels=6)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 7, src, dst, lab)
    og = O.Graph.from_edges(G.V, 7, src, dst, lab)
    rng = np.random.default_rng(12)
    done = 0
    for i in range(30):
        k = int(rng.integers(3, 9))
        q = S.query_random_walk(G, k, rng, tree=bool(i % 3 == 0), bias=1.0 if i % 2 else 0.0)
        if q is None:
            continue
        p = O.plan(q.to_g_text(), enumerate_aut=0)
        try:
            O.match(og, p, limit=3_000_000)
        except O.OracleError:
            continue
        check_case(ctx, g, og, q.to_g_text(), table=True, max_rows=1 << 22)
        done += 1
    assert done >= 6


def test_level_overflow_deferral_gives_identical_results():
    """A tiny SOLN_PREALLOC forces level buffers to fill; chunks are deferred
    and re-run after the deeper levels drain.  Results must not change."""
    G = S.rmat(12, 30000, seed=21, n_elabels=2)
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, 3, src, dst, lab)
    small = fm.Context(prealloc_bytes=256 << 20, soln_prealloc_bytes=24 << 20, output_prealloc_bytes=64 << 20,
                       bank_rows=32)
    g = fm.Graph.from_edges(small, G.V, 3, src, dst, lab)
    q = S.query_path(5, [1, 2, 1, 2])
    p = O.plan(q.to_g_text(), enumerate_aut=0)
    oc = O.match(og, p, count_rule=True)[0]
    for engine in (fm.ENGINE_PERSISTENT, fm.ENGINE_LEVELS):
        r = fm.match(small, g, fm.Query.from_text(q.to_g_text()), mode=fm.MODE_COUNT, engine=engine)
        assert r.count == oc and r.engine == engine
        assert r.passes > p.q - 1 - r.pre_counted     # deferral happened (more passes than launched depths)
    small.close()


def test_table_truncation_keeps_exact_count():
    V, s, d, l = complete_graph(30)
    c = fm.Context(prealloc_bytes=128 << 20, soln_prealloc_bytes=32 << 20, output_prealloc_bytes=1 << 20,
                   bank_rows=32)
    g = fm.Graph.from_edges(c, V, 2, s, d, l)
    q = fm.Query.from_text(S.query_cycle(4, [1] * 4).to_g_text())
    r = fm.match(c, g, q, mode=fm.MODE_TABLE, allow_truncation=True)
    assert r.count == math.perm(30, 4)
    assert r.truncated and r.rows == (1 << 20) // 16
    with pytest.raises(fm.FMError) as ei:
        fm.match(c, g, q, mode=fm.MODE_TABLE)
    assert ei.value.status == fm.FM_ERR_OUTPUT_OVERFLOW
    c.close()


def test_root_ranges_partition_the_count(ctx):
    """Root-range partitioning (the multi-GPU split) sums to the full count."""
    G = S.erdos_renyi(2000, 12000, seed=31, n_elabels=3)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 4, src, dst, lab)
    q = fm.Query.from_text(S.query_cycle(4, [1, 2, 1, 2]).to_g_text())
    full = fm.match(ctx, g, q, mode=fm.MODE_COUNT).count
    cuts = [0, 333, 1000, 1001, 2000]
    parts = [fm.match(ctx, g, q, mode=fm.MODE_COUNT, roots=(a, b)).count for a, b in zip(cuts, cuts[1:])]
    assert sum(parts) == full and full > 0


def test_query_id_columns(ctx):
    G = S.erdos_renyi(300, 1500, seed=2, n_elabels=2)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
    qq = S.query_path(4, [1, 2, 1])
    q = fm.Query.from_text(qq.to_g_text())
    qi = q.info()
    c1, ref_rows, _ = fm.match_table(ctx, g, q, columns=fm.COLUMNS_REFERENCE)
    c2, id_rows, _ = fm.match_table(ctx, g, q, columns=fm.COLUMNS_QUERY_ID)
    assert c1 == c2 > 0
    # reference column i holds the vertex matched at depth q-1-i
    order = [qi.order[d] for d in range(qi.q)]
    perm = [order[qi.q - 1 - i] for i in range(qi.q)]      # original id of each reference column
    conv = np.empty_like(ref_rows)
    conv[:, perm] = ref_rows
    assert np.array_equal(sorted_rows(conv), sorted_rows(id_rows))
    assert all(len(set(r)) == qi.q for r in id_rows.tolist()[:1000])


def test_host_direct_table_matches_device_table(ctx):
    """Rows written straight into pinned host memory equal the device table."""
    G = S.erdos_renyi(3000, 15000, seed=41, n_elabels=2)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
    for qq in (S.query_cycle(4, [1, 2, 1, 2]), S.query_path(5, [1, 1, 2, 2]), S.query_star(3, [1, 2])):
        q = fm.Query.from_text(qq.to_g_text())
        c1, rows1, _ = fm.match_table(ctx, g, q)
        pinned = fm.PinnedRows(c1 + 8, q.q)
        for _ in range(2):
            r = fm.match(ctx, g, q, host_rows=pinned, host_direct=True)
            assert r.count == c1 and r.rows_copied == c1 and r.rows_device is None
            assert np.array_equal(sorted_rows(pinned.view(c1)), sorted_rows(rows1))
        # a too-small host buffer truncates the table, the count stays exact
        small = fm.PinnedRows(max(1, c1 // 3), q.q)
        r = fm.match(ctx, g, q, host_rows=small, host_direct=True, allow_truncation=True)
        assert r.count == c1 and r.truncated == (c1 > small.cap)


def test_single_vertex_and_single_edge_queries(ctx):
    V, s, d, l = cycle_graph(50)
    g = fm.Graph.from_edges(ctx, V, 2, s, d, l)
    one = b"t # 0\n1 0 1 1\nv 0 1\nt # -1"
    r = fm.match(ctx, g, fm.Query.from_text(one), mode=fm.MODE_COUNT)
    assert r.count == 50
    cnt, rows, _ = fm.match_table(ctx, g, fm.Query.from_text(one))
    assert cnt == 50 and sorted(rows[:, 0].tolist()) == list(range(50))
    r = fm.match(ctx, g, fm.Query.from_text(S.query_path(2, [1]).to_g_text()))
    assert r.count == 100


def test_text_and_edge_array_paths_agree(ctx):
    G = S.erdos_renyi(1000, 2000, seed=1, n_elabels=87)
    text = G.to_g_text()
    g1 = fm.Graph.from_text(ctx, text)
    src, dst, lab = G.directed()
    g2 = fm.Graph.from_edges(ctx, G.V, 88, src, dst, lab)
    i1, i2 = g1.info(), g2.info()
    assert (i1.edges, i1.segments, i1.max_list, i1.nbr_words) == (i2.edges, i2.segments, i2.max_list, i2.nbr_words)


@pytest.mark.parametrize("text,status", [
    (b"t # 1\n2 0 1 1\nt # -1", 3),
    (b"t # 0\n2 0 1 1\nt # -2", 4),
    (b"t # 0\n2 x 1 1\nt # -1", 5),
    (b"t # 0\n2 2 1 1\nv 0 1\nv 1 1\ne 0 1 1\nx 1 0 1\nt # -1", 6),
    (b"t # 0\n2 2 1 1\nv 0 1\nv 1 1\ne 0 5 1\ne 1 0 1\nt # -1", 6),
])
def test_data_parser_errors(ctx, text, status):
    with pytest.raises(fm.FMError) as ei:
        fm.Graph.from_text(ctx, text)
    assert ei.value.status == status


def test_graph_cache_loads_the_same_graph(ctx, tmp_path):
    G = S.rmat(12, 20000, seed=61, n_elabels=4)
    p = tmp_path / "d.g"
    p.write_bytes(G.to_g_text())
    c = tmp_path / "d.fmgb"
    fm.write_graph_cache(str(p), str(c))
    a = fm.Graph.from_file(ctx, str(p))
    b = fm.Graph.from_file(ctx, str(c))
    ia, ib = a.info(), b.info()
    for f in ("vertices", "label_slots", "edges", "segments", "long_segments", "max_list", "bitmaps"):
        assert getattr(ia, f) == getattr(ib, f), f
    for qq in (S.query_cycle(4, [1, 2, 3, 4]), S.query_path(5, [1, 1, 2, 3]), S.query_clique(4, [1, 2])):
        q = fm.Query.from_text(qq.to_g_text())
        ca = fm.match(ctx, a, q, mode=fm.MODE_COUNT).count
        assert fm.match(ctx, b, q, mode=fm.MODE_COUNT).count == ca
        if ca <= 1 << 20:
            _, ra, _ = fm.match_table(ctx, a, q, max_rows=1 << 20)
            _, rb, _ = fm.match_table(ctx, b, q, max_rows=1 << 20)
            assert np.array_equal(sorted_rows(ra), sorted_rows(rb))
    a.close()
    b.close()


def test_cli_writes_sorted_table_file(ctx, tmp_path):
    import subprocess
    G = S.erdos_renyi(500, 2500, seed=71, n_elabels=2)
    d = tmp_path / "d.g"
    d.write_bytes(G.to_g_text())
    qt = S.query_cycle(4, [1, 2, 1, 2]).to_g_text()
    qf = tmp_path / "q.g"
    qf.write_bytes(qt)
    out = tmp_path / "t.fmtb"
    env = dict(os.environ, FM_OUTPUT=str(out), FM_OUTPUT_SORTED="1", FM_PREALLOC=str(3 << 30),
               FM_SOLN_PREALLOC=str(1 << 30), FM_OUTPUT_PREALLOC=str(1 << 30))
    r = subprocess.run([os.path.join(os.path.dirname(fm.LIB_PATH), "ForkMatch"), str(qf), str(d)],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    rows, h = fm.read_table(str(out))
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, 3, src, dst, lab)
    oc, orows, _ = O.match(og, O.plan(qt, enumerate_aut=0), table=True, table_cap=1 << 20)
    assert h["sorted"] == 1 and h["rows"] == oc
    assert np.array_equal(rows, sorted_rows(orows))


def _host_parse_status(tmp_path, text):
    p = tmp_path / "h.g"
    p.write_bytes(text)
    try:
        fm.write_graph_cache(str(p), str(tmp_path / "h.fmgb"))
    except fm.FMError as e:
        return e.status, str(e)
    return 0, ""


def test_device_parser_agrees_with_host_parser(ctx, tmp_path):
    """fm_graph_load_text parses on the device; fm_graph_write_cache parses on
    the host.  Same status and message on malformed text, same graph and
    counts on valid text (several blocks of 4 KiB, labels above 255 dropped)."""
    head = b"t # 0\n3 4 1 2\nv 0 1\nv 1 1\nv 2 1\n"
    bad = [
        head + b"e 0 1 1\ne 1 0 1\ne 1 2 2\ne 2 1 2\nt # -1\n",
        head + b"e 0 1 1\ne 1 0 1\ne 1 2 2\ne 2 1 2t # -1",
        head + b"e 0 1 1\ne 1 0 1\ne 1 2 2\ne 2 1 2\ne 0 2 1\nt # -1",
        head + b"e 0 1 1\n\ne 1 0 1\nt # -1",
        head + b"e 0 1 1 \ne 1 0 1\nt # -1",
        head + b"e 0 1 99999999999\nt # -1",
        head + b"e 0 1 3\nt # -1",
        head + b"v 3 1\nt # -1",
        head + b"e 0 1 1\r\nt # -1",
        head + b"e 0 1\nt # -1",
        b"t # 0\n3 4 1 2\n",
    ]
    for text in bad:
        hs, hm = _host_parse_status(tmp_path, text)
        with pytest.raises(fm.FMError) as ei:
            fm.Graph.from_text(ctx, text)
        assert ei.value.status == hs, (text, hm, str(ei.value))
        assert str(ei.value).split("(", 1)[1] == hm.split("(", 1)[1]
    for G in (S.erdos_renyi(20000, 100000, seed=81, n_elabels=300), S.rmat(11, 8000, seed=82, n_elabels=3)):
        text = G.to_g_text()
        assert len(text) > 4 * 4096
        d = fm.Graph.from_text(ctx, text)
        p = tmp_path / "ok.g"
        p.write_bytes(text)
        fm.write_graph_cache(str(p), str(tmp_path / "ok.fmgb"))
        h = fm.Graph.from_file(ctx, str(tmp_path / "ok.fmgb"))
        di, hi = d.info(), h.info()
        for f in ("vertices", "label_slots", "edges", "segments", "long_segments", "max_list", "nbr_words"):
            assert getattr(di, f) == getattr(hi, f), f
        for qq in (S.query_cycle(3, [1, 2, 3]), S.query_path(4, [1, 2, 1]), S.query_star(4, [2, 2, 3])):
            q = fm.Query.from_text(qq.to_g_text())
            assert fm.match(ctx, d, q, mode=fm.MODE_COUNT).count == fm.match(ctx, h, q, mode=fm.MODE_COUNT).count
        d.close()
        h.close()


@pytest.mark.parametrize("data,query,code", [
    (None, b"ok", 12),
    (b"t # 1\n2 0 1 1\nt # -1", b"ok", 76),
    (b"t # 0\n2 0 1 1\nt # -2", b"ok", 77),
    (b"t # 0\n2 x 1 1\nt # -1", b"ok", 78),
    (b"t # 0\n2 2 1 1\nv 0 1\nv 1 1\ne 0 1 1\nx 1 0 1\nt # -1", b"ok", 79),
    (b"ok", None, 232),
    (b"ok", b"t # 0\n2 2 1 1\nv 0 1\nv x 1\ne 0 1 1\ne 1 0 1\nt # -1", 233),
    (b"ok", b"t # 0\n3 2 1 1\nv 0 1\nv 1 1\ne 0 1 1\ne 1 0 1\nt # -1", 234),
    (b"ok", b"t # 0\n4 4 1 1\nv 0 1\nv 1 1\nv 2 1\nv 3 1\ne 0 1 1\ne 1 0 1\ne 2 3 1\ne 3 2 1\nt # -1", 1),
])
def test_cli_exit_codes(tmp_path, data, query, code):
    """The CLI maps every input error to the reference's exit code; the
    oracle's parsers give the same codes for the same texts."""
    import subprocess
    good_data = S.erdos_renyi(50, 120, seed=3, n_elabels=2).to_g_text()
    good_query = S.query_path(3, [1, 2]).to_g_text()
    d = tmp_path / "d.g"
    q = tmp_path / "q.g"
    if data is not None:
        d.write_bytes(good_data if data == b"ok" else data)
    if query is not None:
        q.write_bytes(good_query if query == b"ok" else query)
    env = dict(os.environ, FM_PREALLOC=str(1 << 30), FM_SOLN_PREALLOC=str(256 << 20),
               FM_OUTPUT_PREALLOC=str(256 << 20))
    r = subprocess.run([os.path.join(os.path.dirname(fm.LIB_PATH), "ForkMatch"), str(q), str(d)],
                       capture_output=True, text=True, env=env)
    assert r.returncode == code, r.stdout + r.stderr
    if data not in (None, b"ok"):
        with pytest.raises(O.OracleError) as ei:
            O.Graph.parse(data)
        assert ei.value.code == code
    if query not in (None, b"ok") and code != 1:
        with pytest.raises(O.OracleError) as ei:
            O.plan(query)
        assert ei.value.code == code
