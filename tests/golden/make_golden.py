"""Regenerate the golden fixtures in this folder (run in the build container,
where the ForkMatch sources are present; the GPU machine only reads the output).

ref_planner.json
    For the reference's own query fixtures (dataset/query/*.g, stored verbatim
    as test vectors) and for seeded synthetic queries: the output of the
    reference's host query planner (fileParse + preProcessQuery), obtained by
    running oracle/_ref/ref_planner, which is compiled from the reference
    sources by oracle/build.py.  Fields: matching order as reference
    mappingData, invVertices, per-depth headers (count, index, pkDist,
    lastSymmetry), delta-encoded requirement triples, symmetryCount, |Aut|, or
    the reference's exit code for queries it rejects.

match_cases.json
    Seeded small data graphs (given by generator parameters plus a SHA-256 of
    the generated .g text, so generator drift is caught) with query texts and
    the full embedding count and reference-style count computed by the oracle.

Usage: python tests/golden/make_golden.py
"""
import glob
import hashlib
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from forkmatch_gb300 import synth as S  # noqa: E402
from oracle import build as OB  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF_QUERIES = os.path.join(OB.REF_ROOT, "dataset", "query")


def run_ref_planner(exe, text, timeout=60):
    import tempfile
    with tempfile.NamedTemporaryFile(suffix=".g", delete=False) as f:
        f.write(text)
        path = f.name
    try:
        r = subprocess.run([exe, path], capture_output=True, text=True, timeout=timeout)
    finally:
        os.unlink(path)
    if r.returncode != 0:
        return {"rc": r.returncode}
    return json.loads(r.stdout.strip().splitlines()[-1])


def synthetic_queries():
    rng = np.random.default_rng(20261203)
    out = []
    # fixed shapes, single label (maximally symmetric) and mixed labels
    for k in range(2, 10):
        out.append(("path%d_l1" % k, S.query_path(k, [1] * k)))
        out.append(("star%d_l1" % k, S.query_star(k, [1] * k)))
        if k >= 3:
            out.append(("cycle%d_l1" % k, S.query_cycle(k, [1] * k)))
        if k <= 7:
            out.append(("clique%d_l1" % k, S.query_clique(k, [1])))
        labs = [int(x) for x in rng.integers(1, 3, size=64)]
        out.append(("path%d_l2" % k, S.query_path(k, labs)))
        out.append(("star%d_l2" % k, S.query_star(k, labs)))
        if k >= 3:
            out.append(("cycle%d_l2" % k, S.query_cycle(k, labs)))
        if k <= 7:
            out.append(("clique%d_l2" % k, S.query_clique(k, labs)))
    # random-walk extractions from a small 2-label graph (symmetries appear)
    G = S.erdos_renyi(60, 240, seed=5, n_elabels=2)
    for i in range(40):
        k = int(rng.integers(3, 10))
        q = S.query_random_walk(G, k, rng, tree=bool(i % 3 == 0))
        if q is not None:
            out.append(("walk%d_%d" % (k, i), q))
    # larger queries (q >= 10: symmetryCount forced to 1) with labels
    G2 = S.erdos_renyi(200, 1200, seed=6, n_elabels=16)
    for i in range(12):
        k = int(rng.integers(10, 13))
        q = S.query_random_walk(G2, k, rng, tree=bool(i % 2))
        if q is not None:
            out.append(("big%d_%d" % (k, i), q))
    # queries the reference rejects: disconnected, self loop, missing lines
    out.append(("disconnected", S.Query(4, [(0, 1, 1), (2, 3, 1)])))
    out.append(("selfloop", S.Query(3, [(0, 1, 1), (1, 2, 1), (2, 2, 1)])))
    return out


def main():
    OB.build()
    exe = OB.build_ref_planner()
    if exe is None:
        raise SystemExit("reference sources not found: cannot regenerate ref_planner.json")
    cases = []
    for path in sorted(glob.glob(os.path.join(REF_QUERIES, "*.g"))):
        text = open(path, "rb").read()
        cases.append({"name": "fixture:" + os.path.basename(path), "text": text.decode(),
                      "ref": run_ref_planner(exe, text)})
    for name, q in synthetic_queries():
        text = q.to_g_text()
        cases.append({"name": name, "text": text.decode(), "ref": run_ref_planner(exe, text)})
    # malformed query texts (exit codes of src/hostparser.cuh)
    bad = {
        "bad_prefix": b"t # 1\n2 2 1 1\nv 0 1\nv 1 1\ne 0 1 1\ne 1 0 1\nt # -1",
        "missing_vertex": b"t # 0\n3 2 1 1\nv 0 1\nv 1 1\ne 0 1 1\ne 1 0 1\nt # -1",
        "missing_edge": b"t # 0\n2 4 1 1\nv 0 1\nv 1 1\ne 0 1 1\ne 1 0 1\nt # -1",
        "v_after_e": b"t # 0\n2 2 1 1\nv 0 1\ne 0 1 1\nv 1 1\ne 1 0 1\nt # -1",
    }
    for name, text in bad.items():
        cases.append({"name": name, "text": text.decode(), "ref": run_ref_planner(exe, text)})
    with open(os.path.join(HERE, "ref_planner.json"), "w") as f:
        json.dump(cases, f, indent=0)
    print("ref_planner.json: %d cases" % len(cases))

    # ---- match cases: oracle counts on small seeded graphs
    mcases = []
    graphs = [
        ("er1000_l87", dict(kind="er", n=1000, m=2000, seed=1, n_elabels=87)),
        ("er300_l2", dict(kind="er", n=300, m=1500, seed=2, n_elabels=2)),
        ("er200_l1", dict(kind="er", n=200, m=800, seed=3, n_elabels=1)),
        ("rmat12_l4", dict(kind="rmat", scale=12, m=20000, seed=4, n_elabels=4)),
        ("cl4096_l2", dict(kind="chung_lu", n=4096, m=16000, seed=5, n_elabels=2)),
    ]
    rng = np.random.default_rng(99)
    for gname, params in graphs:
        G = make_graph(params)
        text = G.to_g_text()
        og = O.Graph.parse(text)
        queries = []
        for f in sorted(glob.glob(os.path.join(REF_QUERIES, "*.g"))):
            queries.append(("fixture:" + os.path.basename(f), open(f, "rb").read()))
        for i in range(10):
            k = int(rng.integers(3, 8))
            q = S.query_random_walk(G, k, rng, tree=bool(i % 2))
            if q is not None:
                queries.append((q.name + "_%d" % i, q.to_g_text()))
        shapes = [S.query_cycle(4, [1, 1, 1, 1]), S.query_clique(4, [1]), S.query_star(5, [1, 1, 1, 1]),
                  S.query_path(5, [1, 2, 1, 2])]
        for q in shapes:
            queries.append((q.name, q.to_g_text()))
        entries = []
        for qname, qtext in queries:
            p = O.plan(qtext)
            try:
                full, _, st = O.match(og, p, limit=1 << 32)
            except O.OracleError:
                continue
            if full > 2_000_000:
                continue
            refc = O.ref_count(og, p)
            entries.append({"query": qname, "text": qtext.decode(), "count": int(full), "ref_count": int(refc),
                            "partials": [int(st.partials[d]) for d in range(p.q)],
                            "lookups": [int(st.lookups[d]) for d in range(p.q)],
                            "list_words": [int(st.list_words[d]) for d in range(p.q)]})
        mcases.append({"graph": gname, "params": params, "sha256": hashlib.sha256(text).hexdigest(),
                       "V": G.V, "E": int(og.E), "cases": entries})
        print(gname, len(entries), "cases")
    with open(os.path.join(HERE, "match_cases.json"), "w") as f:
        json.dump(mcases, f, indent=0)


def make_graph(params):
    p = dict(params)
    kind = p.pop("kind")
    if kind == "er":
        return S.erdos_renyi(p["n"], p["m"], p["seed"], p["n_elabels"])
    if kind == "rmat":
        return S.rmat(p["scale"], p["m"], p["seed"], p["n_elabels"])
    if kind == "chung_lu":
        return S.chung_lu(p["n"], p["m"], p["seed"], p["n_elabels"], max_degree=p.get("max_degree", 1 << 20))
    raise ValueError(kind)


if __name__ == "__main__":
    main()
