"""Seeded synthetic data graphs and queries in the ForkMatch ``.g`` format.

Format rules (the ones the reference parser accepts, src/trie.cuh:1075-1097 and
src/hostparser.cuh:286-387): ``t # 0`` line, header ``V E VL EL`` with E = the
number of e-lines, all v-lines before the e-lines, every undirected edge
written as two e-lines with the same label, edge labels 1..EL (the reference
cannot take label 0), Unix line endings and no newline after ``t # -1``.

Generators:
  * ``erdos_renyi``  G(n, m) without duplicates or self loops;
  * ``rmat``         R-MAT(a, b, c, d) with 2^scale vertices, deduplicated, no
                     self loops, vertex ids scrambled by a seeded permutation
                     (the Graph500 convention, so hubs are not all at low ids);
  * ``chung_lu``     power-law expected degrees with a degree cap;
  * queries          random-walk extraction (induced edges, labels copied),
                     spanning trees of a walk, and fixed shapes (path, cycle,
                     star, clique).
"""
import numpy as np


class LabeledGraph:
    """Undirected simple graph: each edge {u, v} (u < v) has one label."""

    def __init__(self, V, u, v, lab, vlab, n_elabels, n_vlabels):
        self.V = int(V)
        self.u = np.asarray(u, dtype=np.uint32)
        self.v = np.asarray(v, dtype=np.uint32)
        self.lab = np.asarray(lab, dtype=np.uint32)
        self.vlab = np.asarray(vlab, dtype=np.uint32)
        self.n_elabels = int(n_elabels)     # labels are 1..n_elabels
        self.n_vlabels = int(n_vlabels)
        self._adj = None

    @property
    def m(self):
        return len(self.u)

    def directed(self):
        """(src, dst, label) with both directions of every edge."""
        src = np.concatenate([self.u, self.v])
        dst = np.concatenate([self.v, self.u])
        lab = np.concatenate([self.lab, self.lab])
        return src, dst, lab

    def adjacency(self):
        if self._adj is None:
            src, dst, lab = self.directed()
            order = np.lexsort((dst, src))
            src, dst, lab = src[order], dst[order], lab[order]
            indptr = np.zeros(self.V + 1, dtype=np.int64)
            np.add.at(indptr, src.astype(np.int64) + 1, 1)
            indptr = np.cumsum(indptr)
            self._adj = (indptr, dst, lab)
        return self._adj

    def to_g_text(self):
        src, dst, lab = self.directed()
        return g_text(self.V, self.vlab, src, dst, lab, self.n_vlabels, self.n_elabels)


# ---------------------------------------------------------------- text writer

def _format_lines(prefix, cols):
    """Vectorised ``prefix c0 c1 ...\\n`` lines for equal-length uint32 columns."""
    n = len(cols[0])
    if n == 0:
        return b""
    cols = [np.asarray(c, dtype=np.uint64) for c in cols]
    ndig = []
    for c in cols:
        d = np.ones(n, dtype=np.int64)
        t = c // 10
        while np.any(t):
            d += (t > 0)
            t //= 10
        ndig.append(d)
    plen = len(prefix)
    linelen = plen + sum(ndig) + len(cols)          # spaces between + final '\n'
    starts = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(linelen, out=starts[1:])
    buf = np.full(int(starts[-1]), ord(" "), dtype=np.uint8)
    pre = np.frombuffer(prefix, dtype=np.uint8)
    for j in range(plen):
        buf[starts[:-1] + j] = pre[j]
    pos = starts[:-1] + plen
    for c, d in zip(cols, ndig):
        x = c.copy()
        end = pos + d - 1
        for j in range(int(d.max())):
            m = d > j
            buf[(end - j)[m]] = (x[m] % 10 + ord("0")).astype(np.uint8)
            x //= 10
        pos = pos + d + 1
    buf[starts[1:] - 1] = ord("\n")
    return buf.tobytes()


def g_text(V, vlab, src, dst, lab, n_vlabels, n_elabels):
    """Whole ``.g`` file as bytes (no newline after ``t # -1``)."""
    head = b"t # 0\n%d %d %d %d\n" % (V, len(src), n_vlabels, n_elabels)
    vl = _format_lines(b"v ", [np.arange(V, dtype=np.uint32), vlab])
    el = _format_lines(b"e ", [src, dst, lab])
    return head + vl + el + b"t # -1"


# ---------------------------------------------------------------- data graphs

def _sorted_unique(a):
    """np.unique for a 1-D integer array, by sort + adjacent compare (much
    faster than np.unique on tens of millions of keys)."""
    a = np.sort(a, kind="stable" if a.dtype.itemsize <= 2 else "quicksort")
    if len(a) == 0:
        return a
    keep = np.empty(len(a), dtype=bool)
    keep[0] = True
    np.not_equal(a[1:], a[:-1], out=keep[1:])
    return a[keep]


def _merge_unique(a, b):
    return _sorted_unique(np.concatenate([a, b]))


def _dedup_pairs(a, b):
    lo = np.minimum(a, b).astype(np.uint64)
    hi = np.maximum(a, b).astype(np.uint64)
    keep = lo != hi
    key = _sorted_unique((lo[keep] << np.uint64(32)) | hi[keep])
    return key


def _finish(V, keys, m, rng, n_elabels, vlab, n_vlabels):
    if len(keys) > m:
        keys = keys[rng.permutation(len(keys))[:m]]
    keys = np.sort(keys)
    u = (keys >> np.uint64(32)).astype(np.uint32)
    v = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    lab = rng.integers(1, n_elabels + 1, size=len(u), dtype=np.uint32)
    return LabeledGraph(V, u, v, lab, vlab, n_elabels, n_vlabels)


def erdos_renyi(n, m, seed, n_elabels, n_vlabels=2, vlabel_base=0):
    """G(n, m): m distinct undirected edges, no self loops, labels 1..n_elabels."""
    rng = np.random.default_rng(seed)
    keys = np.zeros(0, dtype=np.uint64)
    while len(keys) < m:
        k = int((m - len(keys)) * 1.2) + 16
        a = rng.integers(0, n, size=k, dtype=np.uint64)
        b = rng.integers(0, n, size=k, dtype=np.uint64)
        keys = _merge_unique(keys, _dedup_pairs(a, b))
    vlab = rng.integers(vlabel_base, vlabel_base + n_vlabels, size=n, dtype=np.uint32)
    return _finish(n, keys, m, rng, n_elabels, vlab, n_vlabels)


def zipf_labels(rng, n, count, s=1.2, base=1):
    p = 1.0 / np.arange(1, count + 1) ** s
    p /= p.sum()
    return (rng.choice(count, size=n, p=p) + base).astype(np.uint32)


def rmat(scale, m, seed, n_elabels, a=0.57, b=0.19, c=0.19, vlab=None, n_vlabels=1, scramble=True):
    """R-MAT graph with 2^scale vertices and m distinct undirected edges."""
    rng = np.random.default_rng(seed)
    V = 1 << scale
    ab, abc = a + b, a + b + c
    keys = np.zeros(0, dtype=np.uint64)
    while len(keys) < m:
        k = int((m - len(keys)) * 1.15) + 1024
        s = np.zeros(k, dtype=np.uint64)
        t = np.zeros(k, dtype=np.uint64)
        for _ in range(scale):
            r = rng.random(k, dtype=np.float32)
            sb = (r >= ab).astype(np.uint64)                       # quadrants c, d
            tb = (((r >= a) & (r < ab)) | (r >= abc)).astype(np.uint64)   # quadrants b, d
            s = (s << np.uint64(1)) | sb
            t = (t << np.uint64(1)) | tb
        keys = _merge_unique(keys, _dedup_pairs(s, t))
    if scramble:
        perm = rng.permutation(V).astype(np.uint64)
        u = perm[(keys >> np.uint64(32)).astype(np.int64)]
        w = perm[(keys & np.uint64(0xFFFFFFFF)).astype(np.int64)]
        keys = _sorted_unique((np.minimum(u, w) << np.uint64(32)) | np.maximum(u, w))
    if vlab is None:
        vlab = np.ones(V, dtype=np.uint32)
    return _finish(V, keys, m, rng, n_elabels, vlab, n_vlabels)


def chung_lu(n, m, seed, n_elabels, exponent=2.1, max_degree=1 << 20, n_vlabels=1):
    """Chung-Lu graph with power-law expected degrees (capped), deduplicated."""
    rng = np.random.default_rng(seed)
    w = (np.arange(1, n + 1, dtype=np.float64)) ** (-1.0 / (exponent - 1.0))
    w *= 2.0 * m / w.sum()
    w = np.minimum(w, max_degree)
    p = w / w.sum()
    cdf = np.cumsum(p)
    keys = np.zeros(0, dtype=np.uint64)
    rounds = 0
    while len(keys) < m and rounds < 20:
        k = int((m - len(keys)) * 1.3) + 1024
        a = np.searchsorted(cdf, rng.random(k)).astype(np.uint64)
        b = np.searchsorted(cdf, rng.random(k)).astype(np.uint64)
        a = np.minimum(a, n - 1)
        b = np.minimum(b, n - 1)
        keys = _merge_unique(keys, _dedup_pairs(a, b))
        rounds += 1
    perm = rng.permutation(n).astype(np.uint64)
    u = perm[(keys >> np.uint64(32)).astype(np.int64)]
    v = perm[(keys & np.uint64(0xFFFFFFFF)).astype(np.int64)]
    keys = _sorted_unique((np.minimum(u, v) << np.uint64(32)) | np.maximum(u, v))
    vlab = np.ones(n, dtype=np.uint32)
    return _finish(n, keys, m, rng, n_elabels, vlab, n_vlabels)


# ---------------------------------------------------------------- queries

class Query:
    """Small query graph: vertices 0..k-1, undirected labelled edges."""

    def __init__(self, k, edges, vlab=None, name=""):
        self.k = int(k)
        self.edges = [(int(a), int(b), int(l)) for a, b, l in edges]
        self.vlab = list(vlab) if vlab is not None else [1] * self.k
        self.name = name

    @property
    def density(self):
        return len(self.edges) / max(1, self.k * (self.k - 1) // 2)

    def to_g_text(self):
        lines = [b"t # 0", b"%d %d %d %d" % (self.k, 2 * len(self.edges), max(self.vlab + [1]),
                                             max([l for _, _, l in self.edges] + [1]))]
        for i in range(self.k):
            lines.append(b"v %d %d" % (i, self.vlab[i]))
        for a, b, l in self.edges:
            lines.append(b"e %d %d %d" % (a, b, l))
            lines.append(b"e %d %d %d" % (b, a, l))
        lines.append(b"t # -1")
        return b"\n".join(lines)


def query_path(k, labels):
    return Query(k, [(i, i + 1, labels[i]) for i in range(k - 1)], name="path%d" % k)


def query_cycle(k, labels):
    return Query(k, [(i, (i + 1) % k, labels[i]) for i in range(k)], name="cycle%d" % k)


def query_star(k, labels):
    return Query(k, [(0, i, labels[i - 1]) for i in range(1, k)], name="star%d" % k)


def query_clique(k, labels):
    e, t = [], 0
    for i in range(k):
        for j in range(i + 1, k):
            e.append((i, j, labels[t % len(labels)]))
            t += 1
    return Query(k, e, name="clique%d" % k)


def _walk(G, k, rng, bias, max_steps=10000):
    indptr, nbr, lab = G.adjacency()
    deg = np.diff(indptr)
    cand = np.nonzero(deg > 0)[0]
    if bias > 0:
        start = int(rng.choice(cand, p=deg[cand] / deg[cand].sum()))
    else:
        start = int(rng.choice(cand))
    seen = [start]
    pos = {start: 0}
    tree = []
    cur = start
    steps = 0
    while len(seen) < k and steps < max_steps:
        steps += 1
        if bias > 0:
            # frontier of the visited set, weighted by (edges into it)^bias
            fr = {}
            for s in seen:
                for w in nbr[indptr[s]:indptr[s + 1]][:4096]:
                    w = int(w)
                    if w not in pos:
                        fr[w] = fr.get(w, 0) + 1
            if not fr:
                return None
            ws = np.array(list(fr.keys()))
            wt = np.array([fr[x] for x in ws], dtype=np.float64) ** bias
            nxt = int(rng.choice(ws, p=wt / wt.sum()))
            # attach to one visited neighbour for the tree
            par = next(s for s in seen if nxt in set(nbr[indptr[s]:indptr[s + 1]].tolist()))
        else:
            row = nbr[indptr[cur]:indptr[cur + 1]]
            if len(row) == 0:
                return None
            nxt = int(row[rng.integers(0, len(row))])
            par = cur
        if nxt not in pos:
            pos[nxt] = len(seen)
            seen.append(nxt)
            tree.append((par, nxt))
        cur = nxt
    if len(seen) < k:
        return None
    return seen, pos, tree


def _edge_label(G, a, b):
    indptr, nbr, lab = G.adjacency()
    row = nbr[indptr[a]:indptr[a + 1]]
    i = np.searchsorted(row, b)
    if i < len(row) and row[i] == b:
        return int(lab[indptr[a] + i])
    return None


def query_path_walk(G, k, rng, tries=200):
    """Path of k vertices along a random walk of the data graph (labels copied)."""
    indptr, nbr, lab = G.adjacency()
    deg = np.diff(indptr)
    cand = np.nonzero(deg > 0)[0]
    for _ in range(tries):
        cur = int(rng.choice(cand))
        seen = [cur]
        ok = True
        while len(seen) < k:
            row = nbr[indptr[cur]:indptr[cur + 1]]
            fresh = [int(w) for w in row if int(w) not in seen]
            if not fresh:
                ok = False
                break
            cur = fresh[int(rng.integers(0, len(fresh)))]
            seen.append(cur)
        if ok:
            edges = [(i, i + 1, _edge_label(G, seen[i], seen[i + 1])) for i in range(k - 1)]
            q = Query(k, edges, vlab=[int(G.vlab[s]) for s in seen], name="path%d" % k)
            q.source = seen
            return q
    return None


def query_cycle_walk(G, k, rng, tries=200):
    """Cycle of k vertices: a walk path closed by an edge to its start; when the
    data graph has no such edge the closing label is drawn at random (the
    query may then have no match)."""
    p = query_path_walk(G, k, rng, tries)
    if p is None:
        return None
    a, b = p.source[-1], p.source[0]
    lab = _edge_label(G, a, b)
    if lab is None:
        lab = int(rng.integers(1, G.n_elabels + 1))
    q = Query(k, p.edges + [(k - 1, 0, lab)], vlab=p.vlab, name="cycle%d" % k)
    q.source = p.source
    return q


def query_star_sample(G, k, rng, tries=200):
    """Star of k vertices: a centre of degree >= k-1 and k-1 of its neighbours
    (labels copied)."""
    indptr, nbr, lab = G.adjacency()
    deg = np.diff(indptr)
    cand = np.nonzero(deg >= k - 1)[0]
    if len(cand) == 0:
        return None
    for _ in range(tries):
        c = int(rng.choice(cand))
        row = nbr[indptr[c]:indptr[c + 1]]
        leaves = rng.choice(row, size=k - 1, replace=False)
        edges = [(0, i + 1, _edge_label(G, c, int(w))) for i, w in enumerate(leaves)]
        seen = [c] + [int(w) for w in leaves]
        q = Query(k, edges, vlab=[int(G.vlab[s]) for s in seen], name="star%d" % k)
        q.source = seen
        return q
    return None


def query_random_walk(G, k, rng, min_density=0.0, max_density=1.0, tree=False, bias=0.0, tries=200):
    """Query extracted from the data graph by a seeded walk (so >= 1 match).

    tree=False: induced subgraph on the walk's k vertices (labels copied).
    tree=True:  the walk's discovery tree (a spanning tree, labels copied).
    """
    for _ in range(tries):
        w = _walk(G, k, rng, bias)
        if w is None:
            continue
        seen, pos, tr = w
        if tree:
            edges = [(pos[a], pos[b], _edge_label(G, a, b)) for a, b in tr]
        else:
            edges = []
            for i in range(k):
                for j in range(i + 1, k):
                    l = _edge_label(G, seen[i], seen[j])
                    if l is not None:
                        edges.append((i, j, l))
        q = Query(k, edges, vlab=[int(G.vlab[s]) for s in seen])
        if tree or (min_density <= q.density <= max_density):
            q.name = ("tree%d" if tree else "walk%d") % k
            q.source = seen
            return q
    return None


# ---------------------------------------------------------------- large graphs

class BigAdjacency:
    """Neighbour lists of a large LabeledGraph without sorting all e-lines:
    the undirected edges are sorted by u (u < v), so the u-side lists are
    slices, and one argsort of v gives the v-side lists.  Rows are unsorted."""

    def __init__(self, G):
        self.G = G
        idx = np.arange(G.V + 1, dtype=np.int64)
        self.out_ptr = np.searchsorted(G.u, idx)
        order = np.argsort(G.v, kind="stable")
        vs = G.v[order]
        self.in_ptr = np.searchsorted(vs, idx)
        self.in_src = G.u[order]
        self.in_lab = G.lab[order]
        self.deg = np.diff(self.out_ptr) + np.diff(self.in_ptr)

    def neighbours(self, x):
        a, b = self.out_ptr[x], self.out_ptr[x + 1]
        c, d = self.in_ptr[x], self.in_ptr[x + 1]
        return (np.concatenate([self.G.v[a:b], self.in_src[c:d]]),
                np.concatenate([self.G.lab[a:b], self.in_lab[c:d]]))


def query_walk_big(A, k, rng, tries=50):
    """Induced subgraph of a k-vertex random walk (uniform start, uniform
    steps) on a BigAdjacency, labels copied."""
    G = A.G
    for _ in range(tries):
        start = int(rng.integers(0, G.V))
        if A.deg[start] == 0:
            continue
        seen = [start]
        cur = start
        steps = 0
        while len(seen) < k and steps < 30 * k:
            steps += 1
            nb, _ = A.neighbours(cur)
            nxt = int(nb[rng.integers(0, len(nb))])
            if nxt not in seen:
                seen.append(nxt)
            cur = nxt
        if len(seen) < k:
            continue
        edges = []
        for i in range(k):
            nb, lb = A.neighbours(seen[i])
            for j in range(i + 1, k):
                m = nb == seen[j]
                if m.any():
                    edges.append((i, j, int(lb[m][0])))
        q = Query(k, edges, vlab=[int(G.vlab[s]) for s in seen], name="walk%d" % k)
        q.source = seen
        return q
    return None
