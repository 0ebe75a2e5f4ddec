/*
 * forkmatch.h -- C ABI of libforkmatch, a GB300-native (sm_103a) edge-labelled
 * subgraph-isomorphism matcher that is a drop-in for ForkMatch.
 *
 * The reference has no library or FFI: its API surface is the CLI
 * `ForkMatch <query.g> <data.g>` (src/smsm.cu:1351-1393), the .g text format
 * (README.md:5-27), the environment.cuh knobs (src/environment.cuh:4-20) and the
 * embedding table it leaves in device memory (src/smsm.cu:706-779).  Each entry
 * point below names the reference code it replaces.  Plain C types only: no
 * CUDA or torch types appear in the signatures (streams are passed as void*).
 *
 * Semantics (identical to the reference): an embedding is an injective map f
 * from query vertices to data vertices such that for every query e-line
 * (x -> a, label l) with a matched before x, the data graph has an e-line
 * (f(a) -> f(x)) with label l.  Vertex labels are ignored; matches are not
 * induced; duplicate data e-lines yield duplicate embeddings (a value present
 * in every intersected list is produced min(multiplicity) times).
 */
#ifndef FORKMATCH_H
#define FORKMATCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FM_MAX_QUERY_VERTICES 32
#define FM_MAX_LABEL 255

/* Status codes.  Replace the reference's exit()/__trap() error paths
 * (src/trie.cuh:1059-1092, src/hostparser.cuh:15-18,292-387,
 * src/ccsr.cuh:252-254,581-583,719-725, src/tbs.cuh:57-68, src/smsm.cu:898);
 * the CLI maps them back to the reference's exit codes. */
typedef enum fm_status {
    FM_OK = 0,
    FM_ERR_ARG = 1,             /* bad argument */
    FM_ERR_IO = 2,              /* file missing/unreadable            (exit 12 / 232) */
    FM_ERR_DATA_HEADER0 = 3,    /* data text does not start "t # 0\n" (exit 76) */
    FM_ERR_DATA_TRAILER = 4,    /* data text does not end "t # -1"    (exit 77) */
    FM_ERR_DATA_HEADER = 5,     /* malformed data header              (exit 78) */
    FM_ERR_DATA_LINE = 6,       /* malformed/out-of-range data line   (reference traps) */
    FM_ERR_QUERY_FORMAT = 7,    /* malformed query text               (exit 233) */
    FM_ERR_QUERY_MISSING = 8,   /* fewer v/e lines than the header    (exit 234) */
    FM_ERR_DISCONNECTED = 9,    /* query not traversable by the planner (exit 1) */
    FM_ERR_UNSUPPORTED = 10,    /* query outside supported limits */
    FM_ERR_POOL = 11,           /* SOLN_PREALLOC too small for one work chunk */
    FM_ERR_OUTPUT_OVERFLOW = 12,/* table truncated at OUTPUT_PREALLOC (count stays exact) */
    FM_ERR_CUDA = 13,           /* CUDA runtime error (fm_last_error() has the text) */
    FM_ERR_DEVICE = 14,         /* device-side status word reported an error */
    FM_ERR_NOMEM = 15,          /* allocation failed */
    FM_ERR_LIMIT = 16           /* fm_match_opts.work_limit reached (count is a lower bound) */
} fm_status;

const char* fm_status_string(fm_status s);
/* Text of the last error raised on the calling thread. */
const char* fm_last_error(void);

/* Knobs.  Same names and roles as src/environment.cuh:4-20:
 *   PREALLOC       -> prealloc_bytes        (whole device slab of a context)
 *   SOLN_PREALLOC  -> soln_prealloc_bytes   (partial-match levels)
 *   OUTPUT_PREALLOC-> output_prealloc_bytes (embedding table)
 *   CurBankSize    -> bank_rows             (level capacity granularity, rows)
 * fm_knobs_default() gives GB300 defaults, overridden by the environment
 * variables FM_PREALLOC, FM_SOLN_PREALLOC, FM_OUTPUT_PREALLOC, FM_CUR_BANK_SIZE
 * (bytes / rows, decimal). */
typedef struct fm_knobs {
    uint64_t prealloc_bytes;
    uint64_t soln_prealloc_bytes;
    uint64_t output_prealloc_bytes;
    uint32_t bank_rows;
    int32_t device;
} fm_knobs;

void fm_knobs_default(fm_knobs* k);

/* A context owns one device slab (prealloc) and one CUDA stream.  Replaces
 * prealloc()/p_malloc (src/smsm.cu:1171-1180, src/trie.cuh:1029-1049). */
typedef struct fm_context fm_context;
fm_status fm_context_create(const fm_knobs* knobs, fm_context** out);
void fm_context_destroy(fm_context* ctx);
/* cudaStream_t of the context, as void*. */
void* fm_context_stream(fm_context* ctx);

/* Resident data graph: label-partitioned, 16-byte-aligned neighbour segments
 * in device memory.  Replaces parseGraph/parseCSR/csrToTrie and
 * BaseGPUGraph::neighbours (src/trie.cuh:1051-1222, 800-951, 750-795, 266-310).
 * Graph memory is sized to fit at load time (not carved from the slab), so one
 * resident graph serves every context on the same device.  The longest lists
 * also get a bitmap over all vertices (membership in one load instead of a
 * binary search) while the bitmaps fit FM_BITMAP_BYTES (environment, default
 * room for 16384 bitmaps of V bits, within 2..8 GiB; 0 disables) and are at
 * least FM_BITMAP_MIN_LEN (default 64) long;
 * graphs with duplicate e-lines get none. */
typedef struct fm_graph fm_graph;
typedef struct fm_graph_info {
    uint32_t vertices;
    uint32_t label_slots;       /* labels 0 .. label_slots-1 are indexable */
    uint64_t edges;             /* directed e-lines kept */
    uint64_t segments;          /* non-empty (label, vertex) lists */
    uint64_t long_segments;     /* lists stored out of line (length > 3) */
    uint64_t nbr_words;         /* u32 words of out-of-line storage (16 B aligned) */
    uint32_t max_list;          /* longest (label, vertex) list */
    int32_t has_duplicates;     /* some (label, src, dst) e-line occurs twice */
    uint64_t device_bytes;      /* graph bytes resident on the device */
    double build_ms;            /* device build time */
    uint32_t bitmaps;           /* lists that also have a membership bitmap over all vertices */
    uint32_t bitmap_min_len;    /* shortest list given a bitmap (0: none) */
    uint64_t bitmap_bytes;
} fm_graph_info;

/* `.g` file / in-memory text (the reference parser's grammar, README.md:5-27).
 * fm_graph_load_file also takes a binary graph cache (below) at the same path. */
fm_status fm_graph_load_file(fm_context* ctx, const char* path, fm_graph** out);
/* Parse a .g file once and store its e-lines as a binary graph cache
 * ("FMGB0001" header: u32 vertices, u32 label slots, u64 e-lines, u32 label
 * bytes = 1, u32 0; then src[E] u32, dst[E] u32, label[E] u8), which
 * fm_graph_load_file reads without parsing.  Host only, no device. */
fm_status fm_graph_write_cache(const char* text_path, const char* cache_path);
fm_status fm_graph_load_text(fm_context* ctx, const char* text, uint64_t len, fm_graph** out);
/* Directed e-lines from host arrays (both directions must be listed). */
fm_status fm_graph_from_edges(fm_context* ctx, uint32_t vertices, uint32_t label_slots, uint64_t edges,
                              const uint32_t* src, const uint32_t* dst, const uint32_t* label,
                              fm_graph** out);
fm_status fm_graph_get_info(const fm_graph* g, fm_graph_info* info);
void fm_graph_free(fm_graph* g);

/* Compiled query: the reference's matching order and per-depth requirements
 * (src/hostparser.cuh:286-508 fileParse, src/ccsr.cuh:485-728 preProcessQuery,
 * src/ccsr.cuh:229-326 genereateCCSRRequirements) plus its automorphism count
 * (src/ccsr.cuh:383-465 queryMatch). */
typedef struct fm_query fm_query;
typedef struct fm_query_info {
    uint32_t q;                                   /* query vertices */
    uint32_t e_lines;                             /* query e-lines */
    uint32_t max_valency;                         /* longest CCSR row */
    uint32_t order[FM_MAX_QUERY_VERTICES];        /* original vertex id matched at depth d */
    uint32_t local_of_depth[FM_MAX_QUERY_VERTICES];/* reference local (degree-sorted) index at depth d */
    uint32_t inv[FM_MAX_QUERY_VERTICES];          /* reference invVertices: local -> original id */
    uint32_t nreq[FM_MAX_QUERY_VERTICES];         /* back edges per depth */
    uint32_t req_climb[FM_MAX_QUERY_VERTICES][FM_MAX_QUERY_VERTICES];
    uint32_t req_label[FM_MAX_QUERY_VERTICES][FM_MAX_QUERY_VERTICES];
    uint32_t req_refl[FM_MAX_QUERY_VERTICES][FM_MAX_QUERY_VERTICES];
    uint32_t pk_dist[FM_MAX_QUERY_VERTICES];
    uint64_t automorphisms;                       /* |Aut| (label-preserving), 0 if not computed */
} fm_query_info;

fm_status fm_query_compile_file(const char* path, fm_query** out);
fm_status fm_query_compile_text(const char* text, uint64_t len, fm_query** out);
fm_status fm_query_get_info(const fm_query* q, fm_query_info* info);
void fm_query_free(fm_query* q);

/* Matching.  Replaces initPosting/isoInit/isoLoop/isoMatch/isoGen/isInj/
 * attemptInsert/isoWrite and the CDP fork machinery (src/smsm.cu:15-1166)
 * and the host driver match() (src/smsm.cu:1182-1349). */
typedef enum fm_mode {
    FM_MODE_TABLE = 0,          /* count + embedding table (reference WriteSolnFlag = true) */
    FM_MODE_COUNT = 1           /* count only */
} fm_mode;

typedef enum fm_columns {
    FM_COLUMNS_REFERENCE = 0,   /* column i = vertex matched at depth q-1-i (src/smsm.cu:743-760) */
    FM_COLUMNS_QUERY_ID = 1     /* column i = original query vertex i */
} fm_columns;

typedef struct fm_match_opts {
    int32_t mode;               /* fm_mode */
    int32_t columns;            /* fm_columns */
    void* stream;               /* cudaStream_t to run on, or NULL for the context stream */
    uint32_t* host_rows;        /* optional: copy the table here (host memory, pinned preferred) */
    uint64_t host_rows_cap;     /* rows that fit in host_rows */
    uint32_t root_begin;        /* roots (depth-0 images) in [root_begin, root_end); */
    uint32_t root_end;          /*   root_end == 0 means all vertices */
    int32_t profile;            /* 1: time every expansion launch with CUDA events */
    int32_t order;              /* fm_order: matching order used internally */
    int32_t host_direct;        /* 1: the kernels write the table straight into host_rows over
                                   the host link (host_rows must be pinned, e.g. fm_host_alloc);
                                   no device copy of the table is kept */
    uint64_t work_limit;        /* 0: none.  Otherwise stop once more than this many embeddings
                                   were counted, or partial matches produced, and return
                                   FM_ERR_LIMIT (count and rows are then a lower bound) */
    int32_t engine;             /* an fm_engine value, FM_ENGINE_LEVELS by default; profile = 1
                                   always uses FM_ENGINE_LEVELS */
    uint32_t wait_limit_ms;     /* persistent engine: bound on one grid-wide wait between level
                                   passes (0: 60000).  A wait that runs out ends the match with
                                   FM_ERR_DEVICE; the context stays usable */
    int32_t test_stall_barrier; /* tests only: one block never arrives at the first grid
                                   barrier, so every wait of it runs out (checks the bound) */
} fm_match_opts;

/* How the level passes of a match are driven.  Both replace the reference's
 * dynamic-parallelism forks (src/smsm.cu:564-687, 949-1139) and give the same
 * results.
 *   FM_ENGINE_LEVELS (default): one main + heavy launch pair per level pass,
 *     launched back to back; a level whose output buffer filled is drained by
 *     the host, depth first.  Measured faster on GB300 (fewer grid-wide
 *     synchronisations per pass, higher occupancy).
 *   FM_ENGINE_PERSISTENT: one cooperative launch per match.  Each depth has a
 *     device work queue (a ring of chunks pushed back when the output level
 *     filled, then the fresh chunks); the kernel schedules the passes depth
 *     first on the device, and warps that finish their own chunks take pieces
 *     of long (hub) chunks.  No host round trip between passes. */
typedef enum fm_engine {
    FM_ENGINE_LEVELS = 0,
    FM_ENGINE_PERSISTENT = 1
} fm_engine;

/* Matching order.  Results (count, row set, column layout) do not depend on
 * it; only the work does.  FM_ORDER_AUTO picks the order with the smallest
 * estimated partial-match volume for the data graph (cycles closed early);
 * FM_ORDER_REFERENCE uses the reference's greedy order (src/ccsr.cuh:229-326). */
typedef enum fm_order {
    FM_ORDER_AUTO = 0,
    FM_ORDER_REFERENCE = 1
} fm_order;

void fm_match_opts_default(fm_match_opts* o);

typedef struct fm_level_stats {
    uint64_t parents;           /* partial matches expanded at this depth */
    uint64_t lookups;           /* (vertex, label) list lookups */
    uint64_t list_words;        /* sum of looked-up list lengths */
    uint64_t produced;          /* partial matches (or embeddings) produced */
    uint32_t launches;          /* passes of this depth */
    double kernel_ms;           /* sum of launch durations (profile = 1) */
} fm_level_stats;

typedef struct fm_result {
    uint64_t count;             /* exact number of embeddings (u64) */
    uint64_t rows;              /* rows in the device table (min(count, capacity)) */
    const uint32_t* rows_device;/* device table in the context slab; valid until the next match */
    uint64_t rows_copied;       /* rows copied to opts.host_rows */
    int32_t truncated;          /* table capacity exceeded */
    uint32_t q;                 /* row width */
    double device_ms;           /* matching window on the device (CUDA events) */
    uint64_t launches;          /* expansion kernel launches */
    uint64_t h2d_bytes;         /* host->device bytes this match moved (kernel parameter blocks) */
    uint64_t d2h_bytes;         /* device->host bytes (control blocks, totals, copied rows) */
    fm_level_stats level[FM_MAX_QUERY_VERTICES];
    int32_t engine;             /* fm_engine that ran */
    uint32_t passes;            /* level passes over all depths */
    uint64_t max_wait_ns;       /* persistent engine: longest grid-barrier wait of a block */
    int32_t pre_counted;        /* count mode, last depth with one back edge: its extensions were
                                   counted from depth q-2 (its survivors are not stored), so the
                                   last depth was not launched; level[q-1] still reports its work */
    uint32_t reserved;
} fm_result;

fm_status fm_match(fm_context* ctx, const fm_graph* g, const fm_query* q,
                   const fm_match_opts* opts, fm_result* out);

/* Batched matching.  No counterpart in the reference, which matches one query
 * per program run (src/smsm.cu:1182-1349): a batch matches many compiled
 * queries against one resident graph in shared level passes, each query's
 * results identical to fm_match's: max(q) - 1 level launch pairs
 * (FM_ENGINE_LEVELS) or one persistent cooperative launch fed by per-depth
 * work queues (FM_ENGINE_PERSISTENT), captured once as a CUDA graph and
 * replayed.  In table mode the first run counts every query
 * (a counting replay) and then gives each one a table region of exactly its
 * size in OUTPUT_PREALLOC, in batch order while it lasts (a query that does
 * not fit gets FM_ERR_OUTPUT_OVERFLOW; counts stay exact); queries set to
 * count only keep the counts of that counting run and are not matched again
 * in the first run's table pass, and table queries matched alone
 * (fm_batch_set_solo) are matched once, in table mode, each into the free
 * space after the last region.  Queries with one
 * vertex, and every query on a graph with duplicate e-lines, are matched one
 * by one through fm_match (count only). */
typedef struct fm_batch fm_batch;
typedef struct fm_batch_stats {
    uint64_t embeddings;        /* sum of the counts */
    uint64_t launches;          /* kernel launches of the run */
    double wall_ms;             /* host wall time of fm_batch_run */
    uint32_t batched_queries;   /* queries in the shared launches */
    uint32_t single_queries;    /* queries matched one by one */
    uint32_t piece_shift;       /* tuned: split-piece size = base << piece_shift */
    uint32_t grid_quarters;     /* tuned: grid in quarters of the resident blocks per SM */
    uint64_t level_rows;        /* tuned: rows per level buffer (the bank size) */
    int32_t persistent;         /* 1: one cooperative launch per run (FM_ENGINE_PERSISTENT) */
    int32_t graph;              /* 1: the run is a captured CUDA graph replay */
    int32_t weighted_levels;    /* 1: level buffers sized from the previous run's per-depth volumes */
    int32_t solo_queries;       /* tuned: queries matched alone inside the run (the single-query
                                   engine with the whole level memory, table into their region) */
} fm_batch_stats;

fm_status fm_batch_create(fm_context* ctx, const fm_graph* g, const fm_query* const* queries, uint32_t n,
                          int32_t mode, fm_batch** out);
fm_status fm_batch_run(fm_batch* b, uint64_t* counts, fm_batch_stats* stats);
/* Device table of query i after fm_batch_run (table mode): rows of q u32. */
fm_status fm_batch_rows(const fm_batch* b, uint32_t i, const uint32_t** rows_device, uint64_t* rows);
/* Copy query i's table to host memory (up to cap rows). */
fm_status fm_batch_copy_rows(const fm_batch* b, uint32_t i, uint32_t* host, uint64_t cap, uint64_t* copied);
/* Copy every table of the batch to host memory with one device-to-host copy
 * (the regions are packed back to back).  host: cap_words u32.  offsets: n
 * entries (or NULL); offsets[i] = u32 word offset of query i's first row in
 * `host`, UINT64_MAX for a query without a batch table region (matched on its
 * own).  *words = u32 words written.  FM_ERR_OUTPUT_OVERFLOW when cap_words is
 * too small (nothing copied). */
fm_status fm_batch_copy_tables(const fm_batch* b, uint32_t* host, uint64_t cap_words, uint64_t* offsets,
                               uint64_t* words);
/* Query i of a table-mode batch as count only (FM_MODE_COUNT): no table
 * region, its count exact; for queries whose tables cannot be kept.  In count
 * mode a last depth with a single back edge is counted from the list (length
 * minus the vertices already matched) instead of enumerated. */
fm_status fm_batch_set_query_mode(fm_batch* b, uint32_t i, int32_t mode);
/* Engine of later runs: an fm_engine value, FM_ENGINE_LEVELS by default;
 * fm_batch_tune picks the faster one.  Results do not depend on it. */
fm_status fm_batch_set_engine(fm_batch* b, int32_t engine);
/* Query i matched alone inside later runs (solo != 0): on the single-query
 * engine with the whole level memory, after the shared launches, its table
 * in its own region; or back in the shared launches (solo == 0).  Results do
 * not depend on it.  fm_batch_tune picks the queries whose work fills the GPU
 * by themselves; fm_batch_get_solo reads the choice, so that a later batch of
 * the same queries can reuse it without tuning.  Queries matched on their own
 * for other reasons (one vertex, duplicate e-lines) are unaffected. */
fm_status fm_batch_set_solo(fm_batch* b, uint32_t i, int32_t solo);
fm_status fm_batch_get_solo(const fm_batch* b, uint32_t i, int32_t* solo);
/* Autotuner: first times every query alone and keeps the set of queries
 * matched alone (those at or above 8 ms or 2 ms alone, or none) with the
 * fastest run; then runs the batch under each candidate engine, split
 * granularity (the intersection tile a warp walks), grid (warps in flight
 * per SM) and level buffer size (the bank size), keeps the fastest for later
 * runs. */
fm_status fm_batch_tune(fm_batch* b, fm_batch_stats* best);
void fm_batch_free(fm_batch* b);

/* Matching that allocates nothing.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc at match time (an application whose
 * own pool owns all device memory and forbids stray allocations, or a
 * latency-critical loop that cannot afford an allocation).  All scratch lives
 * in one fixed 64 MiB array in this library's device data; a query/graph pair
 * whose partial matches do not fit is rejected with FM_ERR_POOL.  Inputs: a
 * resident graph and a compiled query (q >= 2).  Outputs: *count_out, and --
 * when rows_out is a device buffer of rows_cap rows -- the table in the
 * reference column layout (*rows_written rows; FM_ERR_OUTPUT_OVERFLOW if it did
 * not fit, the count stays exact).  rows_out == NULL counts only.
 * The first call on a device looks up the array's device address; make that
 * first call before any stream capture.  Calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
fm_status fm_match_static(const fm_graph* g, const fm_query* q, uint32_t* rows_out, uint64_t rows_cap,
                          uint64_t* count_out, uint64_t* rows_written, void* stream);

/* Serving: a request loop over one resident graph.  No counterpart in the
 * reference, which matches one query per process (src/smsm.cu:1351-1393).
 * The server takes over the context's PREALLOC slab as its pool: every
 * request leases level buffers (and, in table mode, a table region) sized by
 * its estimated footprint, and is admitted in arrival order as soon as its
 * lease fits the free pool and a slot is idle.  Each slot is one host thread
 * and one stream, so admitted requests overlap on the device; queued
 * count-mode requests are taken together (up to max_batch) and matched in
 * shared level launches (fm_batch).  A footprint that proves too small costs
 * time, never results: level buffers defer and drain, and a truncated table
 * is matched again with an exact lease.  While a server exists, fm_match and
 * fm_batch_create on its context return FM_ERR_ARG. */
typedef struct fm_server fm_server;
typedef struct fm_server_opts {
    uint32_t slots;             /* requests on the device at once; 0 = 4 */
    uint32_t max_batch;         /* count-mode requests matched together; 0 or 1 = one at a time */
    uint64_t min_lease_bytes;   /* smallest level-buffer lease; 0 = pool / (2 * slots), at least 256 MiB */
    uint64_t max_lease_bytes;   /* largest lease of one request; 0 = a quarter of the pool */
    uint64_t work_limit;        /* per request (fm_match_opts.work_limit); 0 = none.  With a
                                   limit, requests are not batched */
} fm_server_opts;
typedef struct fm_serve_result {
    int32_t done;               /* 0 = queued or running */
    fm_status status;
    uint64_t count;
    uint64_t rows_copied;       /* table mode: rows copied to the caller's buffer */
    int32_t truncated;          /* table mode: the caller's buffer was too small */
    uint32_t batch;             /* requests that shared its launches (1 = alone) */
    uint64_t lease_bytes;       /* pool bytes it held (last attempt) */
    uint32_t attempts;          /* runs (a retry follows a lease that was too small) */
    double queue_ms;            /* submit -> admitted */
    double service_ms;          /* admitted -> done */
    double latency_ms;          /* submit -> done */
    char error[128];            /* message of a failed request ("" on success) */
} fm_serve_result;
typedef struct fm_server_stats {
    uint64_t submitted, completed, queued, running;
    uint64_t batches;           /* shared-launch groups run */
    uint64_t embeddings;        /* sum of completed counts */
    uint64_t pool_bytes, pool_free, pool_peak_used;
} fm_server_stats;

fm_status fm_server_create(fm_context* ctx, const fm_graph* g, const fm_server_opts* opts, fm_server** out);
/* Queue a query (copied: it may be freed after the call).  Table mode copies
 * the rows into host_rows (cap rows of q u32; pinned memory copies fastest). */
fm_status fm_server_submit(fm_server* s, const fm_query* q, int32_t mode, uint32_t* host_rows, uint64_t host_rows_cap,
                           uint64_t* ticket);
/* Result of a ticket; wait_ms < 0 waits until done, 0 returns at once.  The
 * result stays available until fm_server_release. */
fm_status fm_server_poll(fm_server* s, uint64_t ticket, int32_t wait_ms, fm_serve_result* out);
fm_status fm_server_release(fm_server* s, uint64_t ticket);
fm_status fm_server_get_stats(fm_server* s, fm_server_stats* out);
/* Finishes every queued request, then stops the slots and returns the slab. */
void fm_server_destroy(fm_server* s);

/* Embedding-table files.  The reference copies its table to the host and
 * drops it (src/smsm.cu:1328-1348); these keep it for parity tooling.
 * File: "FMTB0001", u32 q, u32 columns (fm_columns), u64 rows, u32 sorted,
 * u32 0, then rows x q u32 (little-endian).  sort != 0 writes the rows in
 * lexicographic order, so equal row sets give byte-identical files.  `rows`
 * is host memory in the layout `columns` names. */
fm_status fm_table_write(const char* path, const uint32_t* rows, uint64_t n, uint32_t q, int32_t columns,
                         int32_t sort);
/* Reference column layout -> query-vertex-id layout (column c = image of query
 * vertex c); rows_out may not alias rows_ref. */
fm_status fm_table_to_query_columns(const fm_query* query, const uint32_t* rows_ref, uint64_t n,
                                    uint32_t* rows_out);

/* Pinned host memory helpers (cudaHostAlloc / cudaFreeHost). */
void* fm_host_alloc(uint64_t bytes);
void fm_host_free(void* p);

/* Library / device identification. */
const char* fm_version(void);
int fm_device_count(void);

#ifdef __cplusplus
}
#endif
#endif
