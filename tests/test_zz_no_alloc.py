"""fm_match_static: the entry point for callers that cannot allocate device
memory at match time.  Its scratch is the library's fixed static device array;
its results must equal fm_match's on the same inputs, on two calls in a row
(the array keeps the previous call's contents).  Kept in a file of its own,
collected last."""
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


def test_match_static_equals_fm_match_on_two_calls(setup):
    torch = pytest.importorskip("torch")
    ctx, g = setup
    queries = [S.query_cycle(4, [1, 2, 1, 2]), S.query_path(5, [1, 1, 2, 2]), S.query_star(4, [1, 2, 2]),
               S.query_cycle(3, [1, 1, 2])]
    for qq in queries:
        q = fm.Query.from_text(qq.to_g_text())
        want_count, want_rows, _ = fm.match_table(ctx, g, q)
        assert want_count > 0
        buf = torch.zeros((want_count + 16) * q.q, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        for _ in range(2):
            count, rows = fm.match_static(g, q)                       # count only
            assert (count, rows) == (want_count, 0)
            count, rows = fm.match_static(g, q, rows_device_ptr=buf.data_ptr(), rows_cap=want_count + 16)
            assert count == want_count and rows == want_count
            got = buf[: rows * q.q].cpu().numpy().view(np.uint32).reshape(rows, q.q)
            assert np.array_equal(_sorted(got), _sorted(want_rows))
        # a buffer that is too small: exact count, FM_ERR_OUTPUT_OVERFLOW reported
        count, rows = fm.match_static(g, q, rows_device_ptr=buf.data_ptr(), rows_cap=want_count // 2,
                                      allow_truncation=True)
        assert count == want_count and rows == want_count // 2
