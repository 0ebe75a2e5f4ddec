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


def _label_matrix(G, label):
    """Adjacency matrix of one edge label (both directions), int64 CSR."""
    import scipy.sparse as sp
    src, dst, lab = G.directed()
    m = lab == label
    return sp.csr_matrix((np.ones(int(m.sum()), dtype=np.int64), (src[m].astype(np.int64), dst[m].astype(np.int64))),
                         shape=(G.V, G.V))


def star_count_exact(G, leaf_labels):
    """Exact embedding count of a star whose leaves carry `leaf_labels` on a
    simple graph with one label per edge: sum over centres of the product,
    per label, of the falling factorial of the centre's degree in that label
    (the labels partition a vertex's neighbours, and leaves with the same
    label are an ordered choice of distinct neighbours).  Integer arithmetic;
    raises if a term could overflow int64."""
    src, dst, lab = G.directed()
    total = np.ones(G.V, dtype=np.int64)
    bound = np.ones(G.V, dtype=np.float64)
    for l in sorted(set(leaf_labels)):
        k = leaf_labels.count(l)
        d = np.bincount(src[lab == l], minlength=G.V).astype(np.int64)
        for i in range(k):
            f = np.maximum(d - i, 0)
            total *= f
            bound *= f.astype(np.float64)
    if bound.max() >= 2.0 ** 62 or bound.sum() >= 2.0 ** 63:
        raise OverflowError("star count exceeds int64")
    return int(total.sum())


def path4_count_exact(G, labels):
    """Exact embedding count of the path a-b-c-d with edge labels (l1, l2, l3)
    on a simple graph with one label per edge (no self loops), by inclusion-
    exclusion over the walks a-b-c-d: the walks number
    W = sum over l2-edges (b, c) of d1(b) d3(c); a walk is not injective only
    when a = c (possible only if l1 = l2: c is then an l1-neighbour of b),
    b = d (only if l2 = l3) or a = d (a common l1-neighbour of b and
    l3-neighbour of c: T = sum over l2-edges (b, c) of |N1(b) & N3(c)|); a = c
    together with b = d needs l1 = l2 = l3, and no other two coincide at once
    (they would force a self loop).  So the count is
    W - [l1=l2] sum d3(c) - [l2=l3] sum d1(b) - T + [l1=l2=l3] |E_l2|."""
    l1, l2, l3 = labels
    A1, A2, A3 = _label_matrix(G, l1), _label_matrix(G, l2), _label_matrix(G, l3)
    d1 = np.asarray(A1.sum(axis=1)).ravel().astype(np.int64)
    d3 = np.asarray(A3.sum(axis=1)).ravel().astype(np.int64)
    A2c = A2.tocoo()
    b, c = A2c.row.astype(np.int64), A2c.col.astype(np.int64)
    W = int(np.sum(d1[b] * d3[c]))
    xa = int(np.sum(d3[c])) if l1 == l2 else 0
    xb = int(np.sum(d1[b])) if l2 == l3 else 0
    T = 0
    step = 1 << 16
    for r0 in range(0, G.V, step):
        blk = (A1[r0:r0 + step] @ A3).multiply(A2[r0:r0 + step])
        T += int(blk.sum())
    xab = len(b) if l1 == l2 == l3 else 0
    return W - xa - xb - T + xab


def plain_small_graph():
    p = PLAIN_SMALL
    return S.erdos_renyi(p["n"], p["m"], p["seed"], p["n_elabels"])


def load_workload(name):
    with open(os.path.join(GOLDEN, "workload_%s.json" % name)) as f:
        return json.load(f)
