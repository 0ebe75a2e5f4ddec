"""fm_match_static: the entry point for callers that cannot allocate device
memory at match time.  Its scratch is the library's fixed static device array;
its results must equal fm_match's on the same inputs, on two calls in a row
(the array keeps the previous call's contents), including a match whose
partial-match levels overflow the array's level buffers and are drained
depth first, and it must leave the device's free memory unchanged.  Kept in a
file of its own, collected last."""
import numpy as np
import pytest

import forkmatch_gb300 as fm
from forkmatch_gb300 import synth as S

pytestmark = pytest.mark.gpu


def _sorted(a):
    a = np.asarray(a, dtype=np.uint32)
    return a[np.lexsort(a.T[::-1])] if a.size else a


@pytest.fixture(scope="module")
def setup():
    from forkmatch_gb300 import build
    build.build()
    ctx = fm.Context(prealloc_bytes=1 << 30, soln_prealloc_bytes=256 << 20, output_prealloc_bytes=256 << 20,
                     bank_rows=256)
    G = S.erdos_renyi(3000, 15000, seed=41, n_elabels=2)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 3, src, dst, lab)
    yield ctx, g
    g.close()
    ctx.close()


def _check_twice(ctx, g, q, torch, max_rows=1 << 22):
    want_count, want_rows, _ = fm.match_table(ctx, g, q, max_rows=max_rows)
    assert want_count > 0 and want_rows.shape[0] == want_count
    buf = torch.zeros((want_count + 16) * q.q, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        count, rows = fm.match_static(g, q)                       # count only
        assert (count, rows) == (want_count, 0)
        count, rows = fm.match_static(g, q, rows_device_ptr=buf.data_ptr(), rows_cap=want_count + 16)
        assert count == want_count and rows == want_count
        got = buf[: rows * q.q].cpu().numpy().view(np.uint32).reshape(rows, q.q)
        assert np.array_equal(_sorted(got), _sorted(want_rows))
    return want_count, buf


def test_match_static_equals_fm_match_on_two_calls(setup):
    torch = pytest.importorskip("torch")
    ctx, g = setup
    queries = [S.query_cycle(4, [1, 2, 1, 2]), S.query_path(5, [1, 1, 2, 2]), S.query_star(4, [1, 2, 2]),
               S.query_cycle(3, [1, 1, 2])]
    for qq in queries:
        q = fm.Query.from_text(qq.to_g_text())
        want_count, buf = _check_twice(ctx, g, q, torch)
        # a buffer that is too small: exact count, FM_ERR_OUTPUT_OVERFLOW reported
        count, rows = fm.match_static(g, q, rows_device_ptr=buf.data_ptr(), rows_cap=want_count // 2,
                                      allow_truncation=True)
        assert count == want_count and rows == want_count // 2


def test_match_static_allocates_nothing(setup):
    """After one warm-up call (which loads the library's device code and its
    static array), further calls in both modes leave the device's free memory
    exactly where it was."""
    torch = pytest.importorskip("torch")
    ctx, g = setup
    q = fm.Query.from_text(S.query_cycle(4, [1, 2, 1, 2]).to_g_text())
    want, _ = fm.match_static(g, q)
    buf = torch.zeros((want + 16) * q.q, dtype=torch.int32, device="cuda")
    fm.match_static(g, q, rows_device_ptr=buf.data_ptr(), rows_cap=want + 16)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert fm.match_static(g, q)[0] == want
        assert fm.match_static(g, q, rows_device_ptr=buf.data_ptr(), rows_cap=want + 16) == (want, want)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_match_static_drains_levels_larger_than_its_array():
    """2-paths of a dense single-label graph (7.6 M rows of 3 vertices) do not
    fit the static array's level buffers (about 2.9 M rows for a 4-vertex
    query), so the level is deferred and drained depth first; the count and
    the table still equal fm_match's (whose context holds the level whole)."""
    torch = pytest.importorskip("torch")
    ctx = fm.Context(prealloc_bytes=1 << 30, soln_prealloc_bytes=512 << 20, output_prealloc_bytes=256 << 20,
                     bank_rows=256)
    G = S.erdos_renyi(20000, 200000, seed=43, n_elabels=1)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 2, src, dst, lab)
    q = fm.Query.from_text(S.query_cycle(4, [1, 1, 1, 1]).to_g_text())
    r = fm.match(ctx, g, q, mode=fm.MODE_COUNT, profile=True)
    assert r.level[2].produced > 4_000_000        # the level that overflows the static array
    _check_twice(ctx, g, q, torch)
    g.close()
    ctx.close()


def test_match_static_rejects_a_list_longer_than_its_array_allows():
    """A hub with 30000 neighbours: one 32-parent chunk of an 8-vertex query
    could need more rows than a level buffer of the static array holds, so
    the call is refused up front with FM_ERR_POOL and a zero count."""
    ctx = fm.Context(prealloc_bytes=1 << 30, soln_prealloc_bytes=256 << 20, output_prealloc_bytes=256 << 20,
                     bank_rows=256)
    n = 30001
    G = S.LabeledGraph(n, np.zeros(n - 1, dtype=np.uint32), np.arange(1, n, dtype=np.uint32),
                       np.ones(n - 1, dtype=np.uint32), np.ones(n, dtype=np.uint32), 1, 1)
    src, dst, lab = G.directed()
    g = fm.Graph.from_edges(ctx, G.V, 2, src, dst, lab)
    q = fm.Query.from_text(S.query_path(8, [1] * 7).to_g_text())
    with pytest.raises(fm.FMError) as ei:
        fm.match_static(g, q)
    assert ei.value.status == fm.FM_ERR_POOL
    g.close()
    ctx.close()
