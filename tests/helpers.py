"""Shared helpers for the test suite."""
import hashlib
import json
import os

import numpy as np

from forkmatch_gb300 import synth as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


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


def golden_graphs():
    """Yield (case, LabeledGraph, text) for every graph in match_cases.json,
    checking that the generator still reproduces the recorded bytes."""
    for case in load_golden("match_cases.json"):
        G = make_graph(case["params"])
        text = G.to_g_text()
        assert hashlib.sha256(text).hexdigest() == case["sha256"], "generator drift for " + case["graph"]
        yield case, G, text


def plan_to_ref_format(p):
    """Render an oracle plan the way the reference probe prints it."""
    q, mv = p.q, p.max_valency
    reqs = [[0, 0, 0] for _ in range(mv * q)]
    headers = []
    for d in range(q):
        n = p.nreq[d]
        idx = d * mv * 3
        prev = 0
        for i in range(n):
            c = p.req_climb[d][i]
            reqs[idx // 3 + i] = [c - prev, p.req_label[d][i], p.req_refl[d][i]]
            prev = c
        if n:
            reqs[idx // 3][0] -= 1
        headers.append([n, idx, p.pk_dist[d], p.last_sym[d]])
    return {"rc": 0, "q": q, "max_valency": mv, "sym_count": p.sym_count, "aut_count": p.aut_count,
            "inv": list(p.inv[:q]), "mapping": list(p.ref_mapping[:q]), "headers": headers,
            "reqs": [[x & 0xFFFFFFFF for x in r] for r in reqs]}


def complete_graph(n, label=1):
    src, dst = np.nonzero(~np.eye(n, dtype=bool))
    return n, src.astype(np.uint32), dst.astype(np.uint32), np.full(len(src), label, dtype=np.uint32)


def cycle_graph(n, label=1):
    a = np.arange(n, dtype=np.uint32)
    b = (a + 1) % n
    return n, np.concatenate([a, b]), np.concatenate([b, a]), np.full(2 * n, label, dtype=np.uint32)


def star_graph(d, label=1):
    c = np.zeros(d, dtype=np.uint32)
    leaves = np.arange(1, d + 1, dtype=np.uint32)
    return d + 1, np.concatenate([c, leaves]), np.concatenate([leaves, c]), np.full(2 * d, label, dtype=np.uint32)


def table_sha(rows):
    """SHA-256 of a table's rows sorted lexicographically (u32 little endian)."""
    a = np.asarray(rows, dtype=np.uint32)
    if a.size:
        a = a[np.lexsort(a.T[::-1])]
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def reference_overflows_label_table(n_labels):
    """Whether the reference's graph parser writes one label-graph entry past
    its allocation for a data graph with n_labels edge labels: it allocates
    n_labels + 1 entries of 88 bytes (rounded up to the next multiple of 128
    bytes) and copies n_labels + 1 entries starting at entry 1
    (src/trie.cuh:1115-1138, 1179).  The bytes past the allocation land on the
    presence bitmaps of label 1's first vertices (src/trie.cuh:1162-1166)."""
    size = 88 * (n_labels + 1)
    return 88 > 128 - size % 128


def reference_matches():
    """(graph params, case, reference entry) for every query the reference's
    own GPU build ran (tests/golden/ref_matches.json)."""
    cases = {c["graph"]: {e["query"]: e for e in c["cases"]} for c in load_golden("match_cases.json")}
    out = []
    for g in load_golden("ref_matches.json")["graphs"]:
        for e in g["cases"]:
            if "count" in e:
                out.append((g, cases[g["graph"]][e["query"]], e))
    return out
