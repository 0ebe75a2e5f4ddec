"""forkmatch_gb300 -- Python binding of libforkmatch (GB300-native ForkMatch).

Thin ctypes mirror of ``include/forkmatch.h``.  The library is loaded from
``forkmatch_gb300/lib/libforkmatch.so`` (built in-tree by
``forkmatch_gb300.build``); there is no fallback: if it is missing, importing
``lib()`` raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libforkmatch.so")
CLI_PATH = os.path.join(HERE, "lib", "ForkMatch")
MAXQ = 32

FM_OK = 0
FM_ERR_POOL = 11
FM_ERR_OUTPUT_OVERFLOW = 12
FM_ERR_DEVICE = 14
FM_ERR_LIMIT = 16
MODE_TABLE, MODE_COUNT = 0, 1
COLUMNS_REFERENCE, COLUMNS_QUERY_ID = 0, 1
ORDER_AUTO, ORDER_REFERENCE = 0, 1
ENGINE_LEVELS, ENGINE_PERSISTENT = 0, 1

STATUS_NAMES = {
    0: "FM_OK", 1: "FM_ERR_ARG", 2: "FM_ERR_IO", 3: "FM_ERR_DATA_HEADER0", 4: "FM_ERR_DATA_TRAILER",
    5: "FM_ERR_DATA_HEADER", 6: "FM_ERR_DATA_LINE", 7: "FM_ERR_QUERY_FORMAT", 8: "FM_ERR_QUERY_MISSING",
    9: "FM_ERR_DISCONNECTED", 10: "FM_ERR_UNSUPPORTED", 11: "FM_ERR_POOL", 12: "FM_ERR_OUTPUT_OVERFLOW",
    13: "FM_ERR_CUDA", 14: "FM_ERR_DEVICE", 15: "FM_ERR_NOMEM", 16: "FM_ERR_LIMIT",
}

# Every function include/forkmatch.h declares (checked by the CPU test suite).
EXPORTS = [
    "fm_status_string", "fm_last_error", "fm_knobs_default", "fm_context_create", "fm_context_destroy",
    "fm_context_stream", "fm_graph_load_file", "fm_graph_load_text", "fm_graph_from_edges", "fm_graph_get_info",
    "fm_graph_free", "fm_query_compile_file", "fm_query_compile_text", "fm_query_get_info", "fm_query_free",
    "fm_match_opts_default", "fm_match", "fm_host_alloc", "fm_host_free", "fm_version", "fm_device_count",
    "fm_match_static", "fm_batch_create", "fm_batch_run", "fm_batch_rows", "fm_batch_copy_rows", "fm_batch_tune",
    "fm_batch_free", "fm_batch_copy_tables", "fm_server_create", "fm_server_submit", "fm_server_poll",
    "fm_server_release", "fm_server_get_stats", "fm_server_destroy", "fm_graph_write_cache", "fm_table_write",
    "fm_table_to_query_columns", "fm_batch_set_engine", "fm_batch_set_query_mode", "fm_batch_set_solo",
    "fm_batch_get_solo",
]


class Knobs(ctypes.Structure):
    _fields_ = [("prealloc_bytes", ctypes.c_uint64), ("soln_prealloc_bytes", ctypes.c_uint64),
                ("output_prealloc_bytes", ctypes.c_uint64), ("bank_rows", ctypes.c_uint32),
                ("device", ctypes.c_int32)]


class GraphInfo(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_uint32), ("label_slots", ctypes.c_uint32), ("edges", ctypes.c_uint64),
                ("segments", ctypes.c_uint64), ("long_segments", ctypes.c_uint64), ("nbr_words", ctypes.c_uint64),
                ("max_list", ctypes.c_uint32), ("has_duplicates", ctypes.c_int32), ("device_bytes", ctypes.c_uint64),
                ("build_ms", ctypes.c_double), ("bitmaps", ctypes.c_uint32), ("bitmap_min_len", ctypes.c_uint32),
                ("bitmap_bytes", ctypes.c_uint64)]


_U32Q = ctypes.c_uint32 * MAXQ


class QueryInfo(ctypes.Structure):
    _fields_ = [("q", ctypes.c_uint32), ("e_lines", ctypes.c_uint32), ("max_valency", ctypes.c_uint32),
                ("order", _U32Q), ("local_of_depth", _U32Q), ("inv", _U32Q), ("nreq", _U32Q),
                ("req_climb", _U32Q * MAXQ), ("req_label", _U32Q * MAXQ), ("req_refl", _U32Q * MAXQ),
                ("pk_dist", _U32Q), ("automorphisms", ctypes.c_uint64)]


class MatchOpts(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("columns", ctypes.c_int32), ("stream", ctypes.c_void_p),
                ("host_rows", ctypes.c_void_p), ("host_rows_cap", ctypes.c_uint64),
                ("root_begin", ctypes.c_uint32), ("root_end", ctypes.c_uint32), ("profile", ctypes.c_int32),
                ("order", ctypes.c_int32), ("host_direct", ctypes.c_int32), ("work_limit", ctypes.c_uint64),
                ("engine", ctypes.c_int32), ("wait_limit_ms", ctypes.c_uint32),
                ("test_stall_barrier", ctypes.c_int32)]


class LevelStats(ctypes.Structure):
    _fields_ = [("parents", ctypes.c_uint64), ("lookups", ctypes.c_uint64), ("list_words", ctypes.c_uint64),
                ("produced", ctypes.c_uint64), ("launches", ctypes.c_uint32), ("kernel_ms", ctypes.c_double)]


class Result(ctypes.Structure):
    _fields_ = [("count", ctypes.c_uint64), ("rows", ctypes.c_uint64), ("rows_device", ctypes.c_void_p),
                ("rows_copied", ctypes.c_uint64), ("truncated", ctypes.c_int32), ("q", ctypes.c_uint32),
                ("device_ms", ctypes.c_double), ("launches", ctypes.c_uint64), ("h2d_bytes", ctypes.c_uint64),
                ("d2h_bytes", ctypes.c_uint64), ("level", LevelStats * MAXQ), ("engine", ctypes.c_int32),
                ("passes", ctypes.c_uint32), ("max_wait_ns", ctypes.c_uint64), ("pre_counted", ctypes.c_int32),
                ("reserved", ctypes.c_uint32)]


class BatchStats(ctypes.Structure):
    _fields_ = [("embeddings", ctypes.c_uint64), ("launches", ctypes.c_uint64), ("wall_ms", ctypes.c_double),
                ("batched_queries", ctypes.c_uint32), ("single_queries", ctypes.c_uint32),
                ("piece_shift", ctypes.c_uint32), ("grid_quarters", ctypes.c_uint32),
                ("level_rows", ctypes.c_uint64), ("persistent", ctypes.c_int32), ("graph", ctypes.c_int32),
                ("weighted_levels", ctypes.c_int32), ("solo_queries", ctypes.c_int32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("max_batch", ctypes.c_uint32), ("min_lease_bytes", ctypes.c_uint64),
                ("max_lease_bytes", ctypes.c_uint64), ("work_limit", ctypes.c_uint64)]


class ServeResult(ctypes.Structure):
    _fields_ = [("done", ctypes.c_int32), ("status", ctypes.c_int32), ("count", ctypes.c_uint64),
                ("rows_copied", ctypes.c_uint64), ("truncated", ctypes.c_int32), ("batch", ctypes.c_uint32),
                ("lease_bytes", ctypes.c_uint64), ("attempts", ctypes.c_uint32), ("queue_ms", ctypes.c_double),
                ("service_ms", ctypes.c_double), ("latency_ms", ctypes.c_double), ("error", ctypes.c_char * 128)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("queued", ctypes.c_uint64),
                ("running", ctypes.c_uint64), ("batches", ctypes.c_uint64), ("embeddings", ctypes.c_uint64),
                ("pool_bytes", ctypes.c_uint64), ("pool_free", ctypes.c_uint64), ("pool_peak_used", ctypes.c_uint64)]


_lib = None


def lib():
    """Load libforkmatch.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libforkmatch.so not built: run forkmatch_gb300.build.build() (no fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
        L.fm_status_string.restype = ctypes.c_char_p
        L.fm_status_string.argtypes = [i32]
        L.fm_last_error.restype = ctypes.c_char_p
        L.fm_version.restype = ctypes.c_char_p
        L.fm_knobs_default.argtypes = [ctypes.POINTER(Knobs)]
        L.fm_context_create.argtypes = [ctypes.POINTER(Knobs), ctypes.POINTER(vp)]
        L.fm_context_destroy.argtypes = [vp]
        L.fm_context_stream.argtypes = [vp]
        L.fm_context_stream.restype = vp
        L.fm_graph_load_file.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(vp)]
        L.fm_graph_load_text.argtypes = [vp, ctypes.c_char_p, u64, ctypes.POINTER(vp)]
        L.fm_graph_from_edges.argtypes = [vp, u32, u32, u64, vp, vp, vp, ctypes.POINTER(vp)]
        L.fm_graph_get_info.argtypes = [vp, ctypes.POINTER(GraphInfo)]
        L.fm_graph_free.argtypes = [vp]
        L.fm_query_compile_file.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
        L.fm_query_compile_text.argtypes = [ctypes.c_char_p, u64, ctypes.POINTER(vp)]
        L.fm_query_get_info.argtypes = [vp, ctypes.POINTER(QueryInfo)]
        L.fm_query_free.argtypes = [vp]
        L.fm_match_opts_default.argtypes = [ctypes.POINTER(MatchOpts)]
        L.fm_match.argtypes = [vp, vp, vp, ctypes.POINTER(MatchOpts), ctypes.POINTER(Result)]
        L.fm_host_alloc.argtypes = [u64]
        L.fm_host_alloc.restype = vp
        L.fm_host_free.argtypes = [vp]
        L.fm_match_static.argtypes = [vp, vp, vp, u64, ctypes.POINTER(u64), ctypes.POINTER(u64), vp]
        L.fm_batch_create.argtypes = [vp, vp, ctypes.POINTER(vp), u32, i32, ctypes.POINTER(vp)]
        L.fm_batch_run.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(BatchStats)]
        L.fm_batch_set_engine.argtypes = [vp, i32]
        L.fm_batch_set_query_mode.argtypes = [vp, u32, i32]
        L.fm_batch_set_solo.argtypes = [vp, u32, i32]
        L.fm_batch_get_solo.argtypes = [vp, u32, ctypes.POINTER(i32)]
        L.fm_batch_rows.argtypes = [vp, u32, ctypes.POINTER(vp), ctypes.POINTER(u64)]
        L.fm_batch_copy_rows.argtypes = [vp, u32, vp, u64, ctypes.POINTER(u64)]
        L.fm_batch_copy_tables.argtypes = [vp, vp, u64, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.fm_batch_tune.argtypes = [vp, ctypes.POINTER(BatchStats)]
        L.fm_batch_free.argtypes = [vp]
        L.fm_graph_write_cache.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.fm_table_write.argtypes = [ctypes.c_char_p, vp, u64, u32, i32, i32]
        L.fm_table_to_query_columns.argtypes = [vp, vp, u64, vp]
        L.fm_server_create.argtypes = [vp, vp, ctypes.POINTER(ServerOpts), ctypes.POINTER(vp)]
        L.fm_server_submit.argtypes = [vp, vp, i32, vp, u64, ctypes.POINTER(u64)]
        L.fm_server_poll.argtypes = [vp, u64, i32, ctypes.POINTER(ServeResult)]
        L.fm_server_release.argtypes = [vp, u64]
        L.fm_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
        L.fm_server_destroy.argtypes = [vp]
        _lib = L
    return _lib


class FMError(RuntimeError):
    def __init__(self, status, what):
        msg = lib().fm_last_error().decode(errors="replace")
        super().__init__("%s: %s (%s)" % (what, STATUS_NAMES.get(status, status), msg))
        self.status = status


def _check(st, what, allow=()):
    if st != FM_OK and st not in allow:
        raise FMError(st, what)
    return st


def default_knobs(**overrides):
    k = Knobs()
    lib().fm_knobs_default(ctypes.byref(k))
    for name, v in overrides.items():
        setattr(k, name, v)
    return k


class Context:
    """Device slab + stream (the reference's PREALLOC slab)."""

    def __init__(self, knobs=None, **overrides):
        k = knobs if knobs is not None else default_knobs(**overrides)
        h = ctypes.c_void_p()
        _check(lib().fm_context_create(ctypes.byref(k), ctypes.byref(h)), "fm_context_create")
        self._h = h
        self.knobs = k

    @property
    def stream(self):
        return lib().fm_context_stream(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().fm_context_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Graph:
    """Resident device data graph."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self._h = handle

    @classmethod
    def from_edges(cls, ctx, V, label_slots, src, dst, label):
        src = np.ascontiguousarray(src, dtype=np.uint32)
        dst = np.ascontiguousarray(dst, dtype=np.uint32)
        label = np.ascontiguousarray(label, dtype=np.uint32)
        h = ctypes.c_void_p()
        _check(lib().fm_graph_from_edges(ctx._h, V, label_slots, len(src), src.ctypes.data, dst.ctypes.data,
                                         label.ctypes.data, ctypes.byref(h)), "fm_graph_from_edges")
        return cls(ctx, h)

    @classmethod
    def from_text(cls, ctx, text):
        if isinstance(text, str):
            text = text.encode()
        h = ctypes.c_void_p()
        _check(lib().fm_graph_load_text(ctx._h, text, len(text), ctypes.byref(h)), "fm_graph_load_text")
        return cls(ctx, h)

    @classmethod
    def from_file(cls, ctx, path):
        h = ctypes.c_void_p()
        _check(lib().fm_graph_load_file(ctx._h, os.fsencode(path), ctypes.byref(h)), "fm_graph_load_file")
        return cls(ctx, h)

    def info(self):
        gi = GraphInfo()
        _check(lib().fm_graph_get_info(self._h, ctypes.byref(gi)), "fm_graph_get_info")
        return gi

    def close(self):
        if getattr(self, "_h", None):
            lib().fm_graph_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Query:
    """Compiled query (reference matching order and requirements)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_text(cls, text):
        if isinstance(text, str):
            text = text.encode()
        h = ctypes.c_void_p()
        _check(lib().fm_query_compile_text(text, len(text), ctypes.byref(h)), "fm_query_compile_text")
        return cls(h)

    @classmethod
    def from_file(cls, path):
        h = ctypes.c_void_p()
        _check(lib().fm_query_compile_file(os.fsencode(path), ctypes.byref(h)), "fm_query_compile_file")
        return cls(h)

    def info(self):
        qi = QueryInfo()
        _check(lib().fm_query_get_info(self._h, ctypes.byref(qi)), "fm_query_get_info")
        return qi

    @property
    def q(self):
        return self.info().q

    def close(self):
        if getattr(self, "_h", None):
            lib().fm_query_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


class PinnedRows:
    """Pinned host buffer for embedding rows (fm_host_alloc)."""

    def __init__(self, rows, q):
        self.cap = int(rows)
        self.q = int(q)
        self.ptr = lib().fm_host_alloc(max(1, self.cap * self.q * 4))
        if not self.ptr:
            raise MemoryError("fm_host_alloc failed")
        self.array = np.ctypeslib.as_array(ctypes.cast(self.ptr, ctypes.POINTER(ctypes.c_uint32)),
                                           shape=(max(1, self.cap * self.q),))[: self.cap * self.q]

    def view(self, n):
        return self.array[: n * self.q].reshape(n, self.q)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().fm_host_free(self.ptr)
            self.ptr = None


def match(ctx, graph, query, mode=MODE_TABLE, columns=COLUMNS_REFERENCE, host_rows=None, roots=None,
          profile=False, stream=None, allow_truncation=False, order=ORDER_AUTO, host_direct=False, work_limit=0,
          allow_limit=False, engine=ENGINE_LEVELS, wait_limit_ms=0, test_stall_barrier=False,
          allow_device_error=False):
    """Run fm_match.  Returns the Result struct; with ``host_rows`` (a
    PinnedRows or a C-contiguous uint32 numpy array) the table is copied there.
    ``host_direct`` (PinnedRows only): the kernels write the table straight
    into the pinned host buffer instead of device memory.  ``work_limit``:
    stop after that many embeddings or partial matches (FM_ERR_LIMIT, raised
    unless ``allow_limit``).  ``engine``: ENGINE_LEVELS (launch pairs per
    pass, drains scheduled by the host; the default) or ENGINE_PERSISTENT (one
    cooperative launch, passes scheduled on the device)."""
    o = MatchOpts()
    lib().fm_match_opts_default(ctypes.byref(o))
    o.mode = mode
    o.columns = columns
    o.profile = 1 if profile else 0
    o.order = order
    o.host_direct = 1 if host_direct else 0
    o.work_limit = int(work_limit)
    o.engine = int(engine)
    o.wait_limit_ms = int(wait_limit_ms)
    o.test_stall_barrier = 1 if test_stall_barrier else 0
    if stream is not None:
        o.stream = stream
    if roots is not None:
        o.root_begin, o.root_end = int(roots[0]), int(roots[1])
    if host_rows is not None:
        if isinstance(host_rows, PinnedRows):
            o.host_rows, o.host_rows_cap = host_rows.ptr, host_rows.cap
        else:
            assert host_rows.dtype == np.uint32 and host_rows.flags["C_CONTIGUOUS"]
            o.host_rows = host_rows.ctypes.data
            o.host_rows_cap = host_rows.size // max(1, query.q)
    r = Result()
    st = lib().fm_match(ctx._h, graph._h, query._h, ctypes.byref(o), ctypes.byref(r))
    allow = ((FM_ERR_OUTPUT_OVERFLOW,) if allow_truncation else ()) + ((FM_ERR_LIMIT,) if allow_limit else ()) + \
        ((FM_ERR_DEVICE,) if allow_device_error else ())
    _check(st, "fm_match", allow=allow)
    r.status = st
    return r


class Batch:
    """Many queries against one resident graph in shared level launches
    (fm_batch_*), replayed as a CUDA graph after the first run."""

    def __init__(self, ctx, graph, queries, mode=MODE_COUNT):
        self.ctx, self.graph, self.queries = ctx, graph, list(queries)
        arr = (ctypes.c_void_p * len(self.queries))(*[q._h for q in self.queries])
        h = ctypes.c_void_p()
        _check(lib().fm_batch_create(ctx._h, graph._h, arr, len(self.queries), mode, ctypes.byref(h)),
               "fm_batch_create")
        self._h = h

    def run(self, allow_truncation=False):
        counts = (ctypes.c_uint64 * max(1, len(self.queries)))()
        st = BatchStats()
        s = lib().fm_batch_run(self._h, counts, ctypes.byref(st))
        _check(s, "fm_batch_run", allow=(FM_ERR_OUTPUT_OVERFLOW,) if allow_truncation else ())
        return [int(counts[i]) for i in range(len(self.queries))], st

    def rows(self, i, max_rows):
        q = self.queries[i].q
        buf = np.zeros(max(1, max_rows) * q, dtype=np.uint32)
        n = ctypes.c_uint64()
        _check(lib().fm_batch_copy_rows(self._h, i, buf.ctypes.data, max_rows, ctypes.byref(n)), "fm_batch_copy_rows")
        return buf[: n.value * q].reshape(-1, q)

    def copy_tables(self, host):
        """Copy every table into ``host`` (a PinnedRows or a uint32 numpy
        array) with one device-to-host copy.  Returns (words, offsets):
        offsets[i] is the word offset of query i's rows, or None."""
        n = len(self.queries)
        offs = (ctypes.c_uint64 * max(1, n))()
        words = ctypes.c_uint64()
        if isinstance(host, PinnedRows):
            ptr, cap = host.ptr, host.cap * host.q
        else:
            assert host.dtype == np.uint32 and host.flags["C_CONTIGUOUS"]
            ptr, cap = host.ctypes.data, host.size
        _check(lib().fm_batch_copy_tables(self._h, ptr, cap, offs, ctypes.byref(words)), "fm_batch_copy_tables")
        return words.value, [None if offs[i] == (1 << 64) - 1 else int(offs[i]) for i in range(n)]

    def set_query_mode(self, i, mode):
        _check(lib().fm_batch_set_query_mode(self._h, int(i), int(mode)), "fm_batch_set_query_mode")

    def set_engine(self, engine):
        _check(lib().fm_batch_set_engine(self._h, int(engine)), "fm_batch_set_engine")

    def set_solo(self, i, solo=True):
        """Match query i alone inside later runs (or back in the shared launches)."""
        _check(lib().fm_batch_set_solo(self._h, int(i), 1 if solo else 0), "fm_batch_set_solo")

    def solo(self):
        """Indices of the queries matched alone (chosen by tune() or set_solo)."""
        out = []
        for i in range(len(self.queries)):
            v = ctypes.c_int32()
            _check(lib().fm_batch_get_solo(self._h, i, ctypes.byref(v)), "fm_batch_get_solo")
            if v.value:
                out.append(i)
        return out

    def tune(self):
        st = BatchStats()
        _check(lib().fm_batch_tune(self._h, ctypes.byref(st)), "fm_batch_tune")
        return st

    def close(self):
        if getattr(self, "_h", None):
            lib().fm_batch_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Server:
    """Request loop over a resident graph (fm_server_*): admission by lease
    footprint against the context's slab, slots overlapping on the device,
    count-mode requests batched at the head of the queue."""

    def __init__(self, ctx, graph, slots=4, max_batch=1, min_lease_bytes=0, max_lease_bytes=0, work_limit=0):
        self.ctx, self.graph = ctx, graph
        o = ServerOpts(slots, max_batch, min_lease_bytes, max_lease_bytes, work_limit)
        h = ctypes.c_void_p()
        _check(lib().fm_server_create(ctx._h, graph._h, ctypes.byref(o), ctypes.byref(h)), "fm_server_create")
        self._h = h
        self._keep = {}

    def submit(self, query, mode=MODE_COUNT, host_rows=None):
        """Queue a query; table mode copies rows into ``host_rows`` (a
        PinnedRows or a C-contiguous uint32 array).  Returns the ticket."""
        ptr, cap = None, 0
        if host_rows is not None:
            if isinstance(host_rows, PinnedRows):
                ptr, cap = host_rows.ptr, host_rows.cap
            else:
                assert host_rows.dtype == np.uint32 and host_rows.flags["C_CONTIGUOUS"]
                ptr, cap = host_rows.ctypes.data, host_rows.size // max(1, query.q)
        t = ctypes.c_uint64()
        _check(lib().fm_server_submit(self._h, query._h, mode, ptr, cap, ctypes.byref(t)), "fm_server_submit")
        if host_rows is not None:
            self._keep[t.value] = host_rows
        return t.value

    def poll(self, ticket, wait_ms=-1):
        r = ServeResult()
        _check(lib().fm_server_poll(self._h, ticket, int(wait_ms), ctypes.byref(r)), "fm_server_poll")
        return r

    def release(self, ticket):
        _check(lib().fm_server_release(self._h, ticket), "fm_server_release")
        self._keep.pop(ticket, None)

    def stats(self):
        s = ServerStats()
        _check(lib().fm_server_get_stats(self._h, ctypes.byref(s)), "fm_server_get_stats")
        return s

    def close(self):
        if getattr(self, "_h", None):
            lib().fm_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        self.close()


def write_graph_cache(text_path, cache_path):
    """Parse a .g file once and store it as a binary graph cache, which
    Graph.from_file (fm_graph_load_file) loads without parsing."""
    _check(lib().fm_graph_write_cache(os.fsencode(text_path), os.fsencode(cache_path)), "fm_graph_write_cache")


TABLE_HEADER = np.dtype([("magic", "S8"), ("q", "<u4"), ("columns", "<u4"), ("rows", "<u8"), ("sorted", "<u4"),
                         ("reserved", "<u4")])


def write_table(path, rows, columns=COLUMNS_REFERENCE, sort=True):
    """fm_table_write: rows (n, q) uint32 in the layout ``columns``."""
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    n, q = rows.shape
    _check(lib().fm_table_write(os.fsencode(path), rows.ctypes.data, n, q, columns, 1 if sort else 0),
           "fm_table_write")


def read_table(path):
    """Returns (rows (n, q) uint32, header) of an embedding-table file."""
    with open(path, "rb") as f:
        h = np.frombuffer(f.read(TABLE_HEADER.itemsize), dtype=TABLE_HEADER)[0]
        if h["magic"] != b"FMTB0001":
            raise ValueError("not an embedding-table file")
        rows = np.fromfile(f, dtype="<u4", count=int(h["rows"]) * int(h["q"]))
    return rows.reshape(int(h["rows"]), int(h["q"])), h


def to_query_columns(query, rows_ref):
    """Reference column layout -> query-vertex-id layout."""
    rows_ref = np.ascontiguousarray(rows_ref, dtype=np.uint32)
    out = np.empty_like(rows_ref)
    _check(lib().fm_table_to_query_columns(query._h, rows_ref.ctypes.data, rows_ref.shape[0], out.ctypes.data),
           "fm_table_to_query_columns")
    return out


def match_static(graph, query, rows_device_ptr=None, rows_cap=0, stream=None, allow_truncation=False):
    """fm_match_static: match with no device allocation (scratch in the
    library's fixed static array).  ``rows_device_ptr`` is a device buffer of
    ``rows_cap`` rows of q uint32 (None counts only).  Returns
    (count, rows_written)."""
    cnt = ctypes.c_uint64()
    rows = ctypes.c_uint64()
    st = lib().fm_match_static(graph._h, query._h, rows_device_ptr, int(rows_cap), ctypes.byref(cnt),
                               ctypes.byref(rows), stream)
    _check(st, "fm_match_static", allow=(FM_ERR_OUTPUT_OVERFLOW,) if allow_truncation else ())
    return cnt.value, rows.value


def match_table(ctx, graph, query, columns=COLUMNS_REFERENCE, max_rows=1 << 24, order=ORDER_AUTO):
    """Count and the table as a numpy array (rows copied to host)."""
    q = query.q
    buf = np.zeros(max_rows * q, dtype=np.uint32)
    r = match(ctx, graph, query, mode=MODE_TABLE, columns=columns, host_rows=buf, order=order)
    return r.count, buf[: r.rows_copied * q].reshape(-1, q), r
