"""ctypes wrapper for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and they use it as the checker.  The product library never does.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAXQ = 32


class Plan(ctypes.Structure):
    _fields_ = [
        ("q", ctypes.c_int),
        ("max_valency", ctypes.c_int),
        ("inv", ctypes.c_int * MAXQ),
        ("order", ctypes.c_int * MAXQ),
        ("ref_mapping", ctypes.c_int * MAXQ),
        ("nreq", ctypes.c_int * MAXQ),
        ("req_climb", (ctypes.c_int * MAXQ) * MAXQ),
        ("req_label", (ctypes.c_int * MAXQ) * MAXQ),
        ("req_refl", (ctypes.c_int * MAXQ) * MAXQ),
        ("pk_dist", ctypes.c_int * MAXQ),
        ("last_sym", ctypes.c_int * MAXQ),
        ("aut_count", ctypes.c_uint64),
        ("sym_count", ctypes.c_uint64),
        ("n_edges", ctypes.c_int),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("count", ctypes.c_uint64),
        ("rows_written", ctypes.c_uint64),
        ("partials", ctypes.c_uint64 * MAXQ),
        ("lookups", ctypes.c_uint64 * MAXQ),
        ("list_words", ctypes.c_uint64 * MAXQ),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from oracle import build as _b  # noqa: F401  (build on first use)
            _b.build_oracle()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.ora_graph_from_edges.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                           vp, vp, vp, ctypes.POINTER(vp)]
        L.ora_graph_parse.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(vp)]
        L.ora_graph_free.argtypes = [vp]
        L.ora_graph_vertices.argtypes = [vp]
        L.ora_graph_vertices.restype = ctypes.c_uint32
        L.ora_graph_edges.argtypes = [vp]
        L.ora_graph_edges.restype = ctypes.c_uint64
        L.ora_graph_labels.argtypes = [vp]
        L.ora_graph_labels.restype = ctypes.c_uint32
        L.ora_graph_sources.argtypes = [vp, ctypes.c_uint32]
        L.ora_graph_sources.restype = ctypes.c_uint32
        L.ora_query_plan.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(Plan)]
        L.ora_match.argtypes = [vp, ctypes.POINTER(Plan), ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_int, vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                ctypes.POINTER(Stats)]
        L.ora_match_ex.argtypes = [vp, ctypes.POINTER(Plan), ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                   ctypes.c_int, vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_int, ctypes.POINTER(Stats)]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed with reference exit code %d" % (what, code))
        self.code = code


class Graph:
    """Oracle-side data graph (per-(label, src) sorted lists, duplicates kept)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_edges(cls, V, n_labels, src, dst, label):
        src = np.ascontiguousarray(src, dtype=np.uint32)
        dst = np.ascontiguousarray(dst, dtype=np.uint32)
        label = np.ascontiguousarray(label, dtype=np.uint32)
        h = ctypes.c_void_p()
        rc = lib().ora_graph_from_edges(V, n_labels, len(src), src.ctypes.data, dst.ctypes.data,
                                        label.ctypes.data, ctypes.byref(h))
        if rc:
            raise OracleError(rc, "ora_graph_from_edges")
        return cls(h)

    @classmethod
    def parse(cls, text):
        if isinstance(text, str):
            text = text.encode()
        h = ctypes.c_void_p()
        rc = lib().ora_graph_parse(text, len(text), ctypes.byref(h))
        if rc:
            raise OracleError(rc, "ora_graph_parse")
        return cls(h)

    @property
    def V(self):
        return lib().ora_graph_vertices(self._h)

    @property
    def E(self):
        return lib().ora_graph_edges(self._h)

    def sources(self, label):
        """Vertices with at least one e-line of ``label``."""
        return lib().ora_graph_sources(self._h, int(label))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ora_graph_free(self._h)
            self._h = None


def plan(text, enumerate_aut=None):
    """Reference plan of a query .g text (raises OracleError with the exit code)."""
    if isinstance(text, str):
        text = text.encode()
    p = Plan()
    if enumerate_aut is None:
        enumerate_aut = 1
    rc = lib().ora_query_plan(text, len(text), int(enumerate_aut), ctypes.byref(p))
    if rc:
        raise OracleError(rc, "ora_query_plan")
    return p


def match(graph, p, ref_symmetry=False, roots=None, threads=None, table=False, table_cap=None, limit=0,
          scan_limit=0, count_rule=False):
    """Enumerate embeddings.  Returns (count, rows or None, Stats).
    With ``limit`` > 0, raises OracleError(1000) once the search visited more
    than ``limit`` nodes (partial matches and embeddings); ``scan_limit``
    does the same for the driver-list candidates the nodes scanned.
    ``count_rule`` (count only): a last depth with one requirement is counted
    from its list instead of enumerated (same count)."""
    V = graph.V
    rb, re_ = (0, V) if roots is None else roots
    if threads is None:
        threads = os.cpu_count() or 1
    rows = None
    cap = 0
    if table:
        cap = table_cap if table_cap is not None else 1 << 22
        rows = np.zeros((cap, p.q), dtype=np.uint32)
    st = Stats()
    rc = lib().ora_match_ex(graph._h, ctypes.byref(p), int(bool(ref_symmetry)), rb, re_, int(threads),
                            rows.ctypes.data if rows is not None else None, cap, int(limit), int(scan_limit),
                            int(bool(count_rule)), ctypes.byref(st))
    if rc:
        raise OracleError(rc, "ora_match")
    if rows is not None:
        rows = rows[: st.rows_written]
    return st.count, rows, st


def ref_count(graph, p, threads=None, limit=0):
    """The count the default (SYMMETRY) reference build prints: symmetry-broken
    leaves times symmetryCount when symmetryCount > 1 (src/smsm.cu:724,1305)."""
    c, _, _ = match(graph, p, ref_symmetry=p.sym_count > 1, threads=threads, limit=limit)
    return c * (p.sym_count if p.sym_count > 1 else 1)


def algorithmic_bytes(st, q, V, table=True):
    """Bytes the hot path must move (16 B per (vertex,label) lookup, 4 B per
    list word, 8 B per partial match, 16 B per root lookup, 4q B per row)."""
    b = 16 * V
    for d in range(1, q):
        b += 16 * st.lookups[d] + 4 * st.list_words[d]
    for d in range(q):
        b += 8 * st.partials[d]
    if table:
        b += 4 * q * st.partials[q - 1]
    return b
