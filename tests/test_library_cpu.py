"""The C-ABI library without a GPU: it loads, exports every symbol the header
declares, and its host-side query planner reproduces the reference planner's
recorded output (order, requirements, labels, |Aut|) on the golden cases."""
import os
import re
import subprocess

import pytest

import forkmatch_gb300 as fm
from tests.helpers import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    from forkmatch_gb300 import build
    build.build()


def test_header_declares_exactly_the_exports():
    hdr = open(os.path.join(ROOT, "include", "forkmatch.h")).read()
    declared = set(re.findall(r"\b(fm_[a-z_]+)\s*\(", hdr))
    assert declared == set(fm.EXPORTS)
    L = fm.lib()
    for name in declared:
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", fm.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fm_[a-z_]+)$", out, re.M))
    assert declared <= exported


def test_status_strings_and_version():
    L = fm.lib()
    assert L.fm_status_string(0) == b"ok"
    assert b"sm_103a" in L.fm_version()
    k = fm.default_knobs()
    assert k.soln_prealloc_bytes + k.output_prealloc_bytes < k.prealloc_bytes
    assert k.bank_rows == 1 << 20


def _ref_view(qi):
    """Render the library's plan the way the reference probe prints it."""
    q, mv = qi.q, qi.max_valency
    reqs = [[0, 0, 0] for _ in range(mv * q)]
    headers = []
    for d in range(q):
        n = qi.nreq[d]
        idx = d * mv * 3
        prev = 0
        for i in range(n):
            c = qi.req_climb[d][i]
            reqs[idx // 3 + i] = [c - prev, qi.req_label[d][i], qi.req_refl[d][i]]
            prev = c
        if n:
            reqs[idx // 3][0] -= 1
        headers.append([n, idx, qi.pk_dist[d]])
    mapping = [qi.local_of_depth[q - 1 - i] for i in range(q)]
    return {"q": q, "max_valency": mv, "inv": list(qi.inv[:q]), "mapping": mapping, "headers": headers,
            "reqs": [[x & 0xFFFFFFFF for x in r] for r in reqs]}


# reference exit code -> library status
EXPECTED_STATUS = {1: 9, 233: 7, 234: 8}


@pytest.mark.parametrize("case", load_golden("ref_planner.json"), ids=lambda c: c["name"])
def test_library_planner_matches_reference(case):
    ref = case["ref"]
    try:
        qobj = fm.Query.from_text(case["text"].encode())
    except fm.FMError as e:
        assert ref["rc"] != 0
        if ref["rc"] > 0:
            assert e.status == EXPECTED_STATUS[ref["rc"]]
        return
    assert ref["rc"] == 0
    qi = qobj.info()
    mine = _ref_view(qi)
    want = {k: ref[k] for k in ("q", "max_valency", "inv", "mapping", "reqs")}
    want["headers"] = [h[:3] for h in ref["headers"]]
    assert mine == want
    # |Aut| by orbit-stabiliser equals the reference's brute-force enumeration
    assert qi.automorphisms == ref["aut_count"]
    # matching order in original ids
    assert [qi.order[d] for d in range(qi.q)] == [ref["inv"][ref["mapping"][qi.q - 1 - d]] for d in range(qi.q)]


def test_large_symmetric_query_aut_count_is_fast():
    from forkmatch_gb300 import synth as S
    import math
    q = fm.Query.from_text(S.query_star(16, [1] * 15).to_g_text())
    assert q.info().automorphisms == math.factorial(15)
    q = fm.Query.from_text(S.query_cycle(16, [1] * 16).to_g_text())
    assert q.info().automorphisms == 32


def test_cli_wrong_argument_count_exits_99():
    r = subprocess.run([fm.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 99
    assert r.stdout.startswith("Trie Graph Problem")


def test_graph_cache_holds_the_parsed_e_lines(tmp_path):
    """fm_graph_write_cache parses a .g file once; its e-lines equal the ones
    in the text (the oracle's parser reads the same text)."""
    from forkmatch_gb300 import synth as S
    G = S.erdos_renyi(300, 900, seed=5, n_elabels=7)
    text = G.to_g_text()
    p = tmp_path / "data.g"
    p.write_bytes(text)
    c = tmp_path / "data.fmgb"
    fm.write_graph_cache(str(p), str(c))
    raw = c.read_bytes()
    assert raw[:8] == b"FMGB0001"
    import numpy as np
    V, L = np.frombuffer(raw[8:16], dtype="<u4")
    E = int(np.frombuffer(raw[16:24], dtype="<u8")[0])
    src, dst, lab = G.directed()
    assert (V, E) == (300, len(src)) and L == 8
    body = raw[32:]
    assert len(body) == 9 * E
    cs = np.frombuffer(body[: 4 * E], dtype="<u4")
    cd = np.frombuffer(body[4 * E: 8 * E], dtype="<u4")
    cl = np.frombuffer(body[8 * E:], dtype=np.uint8)
    got = sorted(zip(cs.tolist(), cd.tolist(), cl.tolist()))
    assert got == sorted(zip(src.tolist(), dst.tolist(), lab.tolist()))
    with pytest.raises(fm.FMError):
        fm.write_graph_cache(str(tmp_path / "missing.g"), str(c))


def test_table_files_sorted_and_in_query_columns(tmp_path):
    import numpy as np
    rng = np.random.default_rng(3)
    rows = rng.integers(0, 50, size=(5000, 4)).astype(np.uint32)
    p = tmp_path / "t.fmtb"
    fm.write_table(str(p), rows, sort=True)
    got, h = fm.read_table(str(p))
    assert h["q"] == 4 and h["rows"] == 5000 and h["sorted"] == 1 and h["columns"] == fm.COLUMNS_REFERENCE
    assert np.array_equal(got, rows[np.lexsort(rows.T[::-1])])
    fm.write_table(str(p), rows, sort=False)
    assert np.array_equal(fm.read_table(str(p))[0], rows)
    # reference layout: column i = image of the vertex matched at depth q-1-i
    from forkmatch_gb300 import synth as S
    q = fm.Query.from_text(S.query_path(4, [1, 2, 3]).to_g_text())
    info = q.info()
    out = fm.to_query_columns(q, rows)
    for i in range(4):
        assert np.array_equal(out[:, info.order[4 - 1 - i]], rows[:, i])
