"""Record the query sets of the benchmark workloads (run in the build container).

workload_plain_at_scale.json
    Graph: forkmatch_gb300.workloads.plain_at_scale_graph() (its edge-array
    SHA-256 is stored).  Queries: seeded random walks of 8 vertices with
    induced edges and copied labels.
      * 8 "dense" queries: induced edge density >= 0.5;
      * 8 "sparse" queries: density in [0.40, 0.50).
    The configuration's other half, 8 spanning trees of a walk, is not
    enumerable: on this graph such trees have about 10^16 embeddings each (a
    homomorphism count by sparse matrix-vector products bounds it), and so do
    walks of density <= 0.39 (> 4e9 within seconds).  The sparsest band whose
    counts fit a uint32 table stands in for them.  A candidate is kept when the
    oracle's full count is at most 2^28 (the table then fits in 8.6 GB).
    Counts are the oracle's exact full counts, so the benchmark doubles as a
    full-size bit-exact check.

Usage: python tests/golden/make_workloads.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import numpy as np  # noqa: E402

from forkmatch_gb300 import synth as S  # noqa: E402
from forkmatch_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

LIMIT = 1 << 28


def main():
    t0 = time.time()
    G = W.plain_at_scale_graph()
    src, dst, lab = G.directed()
    og = O.Graph.from_edges(G.V, G.n_elabels + 1, src, dst, lab)
    print("graph %.1fs" % (time.time() - t0), flush=True)
    rng = np.random.default_rng(20261203)
    picked = {"dense": [], "sparse": []}
    bands = {"dense": (0.5, 1.0, 3.0), "sparse": (0.40, 0.4999, 2.0)}
    attempts = 0
    while min(len(v) for v in picked.values()) < 8 and attempts < 200:
        attempts += 1
        for kind, (lo, hi, bias) in bands.items():
            if len(picked[kind]) >= 8:
                continue
            q = S.query_random_walk(G, 8, rng, min_density=lo, max_density=hi, bias=bias, tries=400)
            if q is None:
                continue
            text = q.to_g_text()
            p = O.plan(text, enumerate_aut=0)
            t = time.time()
            try:
                c, _, st = O.match(og, p, limit=LIMIT)
            except O.OracleError:
                print(kind, "rejected (count > 2^28)", flush=True)
                continue
            if c == 0:
                continue
            picked[kind].append({"kind": kind, "text": text.decode(), "edges": len(q.edges),
                                 "density": round(q.density, 4), "count": int(c),
                                 "oracle_seconds": round(time.time() - t, 3)})
            print(kind, len(q.edges), "count", c, "%.2fs" % (time.time() - t), flush=True)
    out = {"workload": "plain_at_scale", "params": W.PLAIN_AT_SCALE, "V": G.V, "E": int(len(src)),
           "edge_sha256": W.edge_hash(src, dst, lab),
           "queries": picked["dense"] + picked["sparse"]}
    with open(os.path.join(HERE, "workload_plain_at_scale.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("total embeddings", sum(q["count"] for q in out["queries"]), "%.1fs" % (time.time() - t0))


if __name__ == "__main__":
    main()
