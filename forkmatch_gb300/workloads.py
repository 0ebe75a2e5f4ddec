"""Synthetic workloads with the shapes of the benchmark configurations.

Every graph is generated from a fixed seed by ``forkmatch_gb300.synth``; the
edge arrays are hashed so a run can tell whether its generator reproduced the
recorded graph exactly.

plain_at_scale (the headline workload):
    R-MAT(a=0.57, b=0.19, c=0.19, d=0.05), 2^20 vertices, 16M distinct
    undirected edges without self loops (32M directed e-lines), vertex labels
    Zipf(s=1.2) over 4 values (ignored by matching, as in the reference), edge
    labels uniform over 32 (written 1..32), uint32 ids.  16 queries of 8
    vertices, matched one at a time with full uint32 embedding tables.
    The query set is recorded in tests/golden/workload_plain_at_scale.json.

batched (the multi-query workload):
    R-MAT(0.57, 0.19, 0.19, 0.05), 2^22 vertices, 64M distinct undirected
    edges (128M directed e-lines), vertex labels uniform over 8, edge labels
    uniform over 64, uint32 ids.  512 queries of 4-16 vertices (size uniform)
    and mixed shape: paths, cycles, stars and random-walk-induced subgraphs of
    edge density 0.3-0.8, each drawn from the graph with copied labels.  The
    query set with per-query counts is recorded in
    tests/golden/workload_batched.json.

skew (the stress workload for level buffers and work splitting):
    Chung-Lu, 2^21 vertices, power-law exponent 2.1, expected degrees capped
    at 2^20, 32M distinct undirected edges, one vertex label, 2 edge labels;
    5-vertex stars, 4-cycles and 4-cliques, count only (u64).

serving (the request-loop workload):
    R-MAT(0.57, 0.19, 0.19, 0.05), 2^24 vertices, 256M distinct undirected
    edges (512M directed e-lines), vertex labels uniform over 8, edge labels
    uniform over 64, uint32 ids, resident on the device.  Queries of 4-12
    vertices are induced subgraphs of seeded random walks, screened on the
    device (a root sample first, then the full count) so that every request
    is an interactive one; arrivals are Poisson at swept rates.
"""
import hashlib
import json
import os

import numpy as np

from forkmatch_gb300 import synth as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")

PLAIN_AT_SCALE = dict(scale=20, m=16_000_000, n_elabels=32, n_vlabels=4, seed=2, vlabel_seed=3)
PLAIN_SMALL = dict(n=1000, m=2000, n_elabels=87, seed=1)
BATCHED = dict(scale=22, m=64_000_000, n_elabels=64, n_vlabels=8, seed=5, vlabel_seed=6)
SERVING = dict(scale=24, m=256_000_000, n_elabels=64, n_vlabels=8, seed=7, vlabel_seed=8)
SKEW = dict(n=1 << 21, m=32_000_000, n_elabels=2, exponent=2.1, max_degree=1 << 20, seed=9)


def edge_hash(src, dst, lab):
    h = hashlib.sha256()
    for a in (src, dst, lab):
        h.update(np.ascontiguousarray(a, dtype=np.uint32).tobytes())
    return h.hexdigest()


def plain_at_scale_graph():
    p = PLAIN_AT_SCALE
    rng = np.random.default_rng(p["vlabel_seed"])
    vlab = S.zipf_labels(rng, 1 << p["scale"], p["n_vlabels"], s=1.2)
    return S.rmat(p["scale"], p["m"], p["seed"], p["n_elabels"], vlab=vlab, n_vlabels=p["n_vlabels"])


def batched_graph():
    p = BATCHED
    rng = np.random.default_rng(p["vlabel_seed"])
    vlab = rng.integers(0, p["n_vlabels"], size=1 << p["scale"], dtype=np.uint32)
    return S.rmat(p["scale"], p["m"], p["seed"], p["n_elabels"], vlab=vlab, n_vlabels=p["n_vlabels"])


def serving_graph(scale=None, m=None):
    p = dict(SERVING)
    if scale is not None:
        p["scale"], p["m"] = scale, m
    rng = np.random.default_rng(p["vlabel_seed"])
    vlab = rng.integers(0, p["n_vlabels"], size=1 << p["scale"], dtype=np.uint32)
    return S.rmat(p["scale"], p["m"], p["seed"], p["n_elabels"], vlab=vlab, n_vlabels=p["n_vlabels"])


def skew_graph():
    p = SKEW
    return S.chung_lu(p["n"], p["m"], p["seed"], p["n_elabels"], exponent=p["exponent"], max_degree=p["max_degree"])


def star_count_closed_form(G, leaf_labels):
    """Embeddings of a star whose leaves carry `leaf_labels`: sum over centres
    of the product, per label, of the falling factorial of the centre's
    degree in that label (labels partition a vertex's neighbours).  Float:
    the value can exceed 2^64."""
    src, dst, lab = G.directed()
    total = np.ones(G.V)
    for l in sorted(set(leaf_labels)):
        k = leaf_labels.count(l)
        d = np.bincount(src[lab == l], minlength=G.V).astype(np.float64)
        f = np.ones(G.V)
        for i in range(k):
            f *= np.maximum(d - i, 0)
        total *= f
    return float(total.sum())


def plain_small_graph():
    p = PLAIN_SMALL
    return S.erdos_renyi(p["n"], p["m"], p["seed"], p["n_elabels"])


def load_workload(name):
    with open(os.path.join(GOLDEN, "workload_%s.json" % name)) as f:
        return json.load(f)
