// fm_internal.h -- shared internals of libforkmatch (host + device).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "forkmatch.h"

namespace fm {

constexpr int kMaxQ = FM_MAX_QUERY_VERTICES;
constexpr int kMaxReqTotal = 512;       // back edges over all depths of one query
constexpr uint32_t kBitmapMark = 0x80000000u;   // long record: z holds a bitmap index
constexpr uint32_t kNoVertex = 0xffffffffu;

// Thread-local error text (fm_last_error).
void set_error(const std::string& msg);
fm_status cuda_fail(cudaError_t e, const char* what);

#define FM_CUDA(call)                                              \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ::fm::cuda_fail(_e, #call); \
    } while (0)

#define FM_TRY(call)                       \
    do {                                   \
        fm_status _s = (call);             \
        if (_s != FM_OK) return _s;        \
    } while (0)

// ----------------------------------------------------------------- data graph
// Segment record of one (label, vertex) list, one 16-byte load per lookup:
//   len <= 3 : {len, n0, n1, n2}      neighbours inline, unused slots 0xffffffff
//   len >  3 : {len, off16, min, max} list at nbr[off16*4 .. off16*4+len), 16-B aligned
struct DeviceGraph {
    uint32_t V = 0;
    uint32_t L = 0;            // label slots
    uint32_t vbits = 0;        // bits per vertex id in the sort key
    uint64_t E = 0;
    uint4* seg = nullptr;      // L*V records, index label*V + v
    uint32_t* nbr = nullptr;   // out-of-line lists
    // Source vertex of every non-empty segment, label-major: the vertices with
    // at least one e-line of label l are heads[head_off[l] .. head_off[l+1]),
    // ascending.  A matching's roots come from the list of a depth-1 label.
    uint32_t* heads = nullptr;
    std::vector<uint64_t> head_off;      // L + 1 entries (host)
    // Membership bitmaps of the longest lists: a long record whose z field
    // has kBitmapMark set keeps its bitmap (bm_words u32 over all vertices) at
    // bitmaps + (z & ~kBitmapMark) * bm_words instead of its minimum.
    uint32_t* bitmaps = nullptr;
    uint32_t bm_words = 0;
    uint32_t n_bitmaps = 0;
    uint32_t bm_min_len = 0;
    uint64_t nbr_words = 0;
    uint64_t segments = 0, long_segments = 0;
    uint32_t max_len = 0;
    int has_dups = 0;
    int has_self_loops = 0;    // some e-line has src == dst
    int device = 0;
    double build_ms = 0;
    std::vector<uint64_t> label_count;   // e-lines per label slot
};

// ----------------------------------------------------------------- query plan
struct LocalELine {
    uint32_t a, b, l;                    // local a -> local b with label l
};

struct Plan {
    uint32_t q = 0;
    uint32_t e_lines = 0;
    uint32_t max_valency = 0;
    uint32_t inv[kMaxQ] = {};            // local -> original id
    uint32_t order_local[kMaxQ] = {};    // reference matching order: depth -> local index
    uint32_t nreq[kMaxQ] = {};
    uint32_t req_climb[kMaxQ][kMaxQ] = {};
    uint32_t req_label[kMaxQ][kMaxQ] = {};
    uint32_t req_refl[kMaxQ][kMaxQ] = {};
    uint32_t pk_dist[kMaxQ] = {};
    uint64_t automorphisms = 0;
    // e-lines of every local row, each row ordered by neighbour (the CCSR rows)
    std::vector<LocalELine> rows;
};

// Device-side copy of a plan, passed by value to every expansion launch.
struct DevPlan {
    uint32_t q;
    uint32_t nreq[kMaxQ];
    uint32_t req_begin[kMaxQ];
    uint8_t req_anc[kMaxReqTotal];     // ancestor depth (row column) of each requirement
    uint8_t req_label[kMaxReqTotal];
    uint8_t out_col[kMaxQ];            // table column of the vertex matched at depth d
    uint8_t col_depth[kMaxQ];          // depth whose vertex fills table column c
};

// Requirements of an arbitrary matching order (the reference's rule applied to
// `order`): at depth d, the e-lines of the new vertex's row to vertices matched
// earlier, ordered by climb.  Returns false if some depth >= 1 has none.
bool order_requirements(const Plan& P, const uint32_t* order, uint32_t nreq[kMaxQ],
                        uint32_t climb[kMaxQ][kMaxQ], uint32_t label[kMaxQ][kMaxQ]);
// Cost-based matching order for a data graph (fm_parse.cpp).
void choose_order(const Plan& P, const DeviceGraph& g, uint32_t order[kMaxQ]);

// Per-launch control block in device memory.
struct LaunchCtl {
    unsigned long long claim;       // work items claimed
    unsigned long long budget;      // output rows reserved (upper bound)
    unsigned long long produced;    // output rows written (exact)
    unsigned long long parents;
    unsigned long long lookups;
    unsigned long long list_words;
    unsigned int stop;              // level buffer full: stop claiming
    unsigned int ndef;              // deferred chunks written
    unsigned int error;
    unsigned int pad;
    unsigned long long heavy;       // heavy chunks: (entries << 32) | pieces, one packed atomic
    unsigned long long claim2;      // heavy pieces claimed
};

// A chunk whose candidate range is too long for one warp: its slots are cut
// into pieces of kHeavyPiece and spread over every warp of a second launch.
struct HeavyEntry {
    uint32_t chunk;
    uint32_t total;                 // candidate slots of the chunk
    uint32_t piece0;                // first global piece index
    uint32_t pieces;
};

// Per-match totals in device memory.
struct MatchTotals {
    unsigned long long count;       // embeddings (last level)
    unsigned long long table_pos;   // rows reserved in the table
    unsigned int error;
    unsigned int pad[3];
};

enum KernelMode { kModeMid = 0, kModeLastTable = 1, kModeLastCount = 2 };

struct ExpandParams {
    DevPlan plan;
    // graph
    const uint4* seg;
    const uint32_t* nbr;
    const uint32_t* bm;             // list bitmaps (see DeviceGraph)
    uint32_t bm_words;
    uint32_t V;
    // parents
    const uint32_t* pin;            // SoA: column c at pin + c*pstride (null for roots)
    uint64_t pstride;
    uint64_t n_parents;
    // when set, n_parents is read on the device from here (the previous level's
    // `produced`) and the launch covers fresh chunks only: levels can then be
    // launched back to back without the host reading anything in between
    const unsigned long long* n_parents_dev;
    uint32_t root_begin;            // roots: parent p is vertex root_begin + p
    const uint32_t* root_list;      // roots, when set: parent p is vertex root_list[p]
    uint32_t depth;                 // parent rows have `depth` entries; new vertex goes to column depth
    // work items: ndef_in deferred chunks, then fresh chunks from fresh_base.
    // Deferred lists are rings of def_cap entries: deferred item i is
    // def_in[(def_in_pos + i) % def_cap]; a new deferral goes to
    // def_out[(def_out_pos + k) % def_cap] while k < def_room.  The level-launch
    // driver uses two plain lists (positions 0, room def_cap); the persistent
    // kernel keeps one ring per depth (def_in == def_out).
    const uint32_t* def_in;
    uint32_t ndef_in;
    uint64_t fresh_base;            // first fresh chunk
    uint64_t n_items;               // ndef_in + fresh chunks
    uint32_t* def_out;
    uint32_t def_cap;
    uint64_t def_in_pos;
    uint64_t def_out_pos;
    uint32_t def_room;
    // outputs
    uint32_t* pout;                 // SoA, column c at pout + c*ocap
    uint64_t ocap;
    uint32_t* table;                // rows of q (device memory, or mapped pinned host memory)
    uint64_t table_cap;
    uint32_t table_vec4;            // rows can be written as 16-byte vectors (q % 4 == 0, aligned)
    LaunchCtl* ctl;
    MatchTotals* tot;
    HeavyEntry* heavy;
    uint32_t heavy_cap;             // entries; chunks are published only while room remains
    uint32_t max_warps;             // warps of the heavy pass (bounds concurrent publishers)
    // last level: stop once the count (or reserved table rows) exceeds this,
    // setting bit kLimitFlag in tot->error; 0 = no limit
    unsigned long long work_limit;
    // words of each warp's shared-memory stage for membership lists copied in
    // by TMA (levels with two or more back edges); 0 = lists are searched in
    // global memory
    uint32_t stage_words;
    // Count mode, the query's last depth has one back edge (no duplicate
    // e-lines): the counting level is depth q-2, whose survivors are not
    // stored but counted by their extensions (the single list's length minus
    // the row's vertices found in it); depth q-1 is never launched.  Its work
    // counters (parents, lookups, list words) are added to ctl[1] of the
    // counting level's control block array (the next depth's block).
    uint32_t pre_count;
    // The graph has an e-line v -> v: only then can a vertex be in its own
    // list, so only then does pre-count test the new vertex against its list.
    uint32_t self_loops;
};
constexpr unsigned int kLimitFlag = 2u;

// ------------------------------------------------------- persistent engine
// One cooperative launch runs every level pass of a match: each pass is the
// main pass, a grid barrier, the heavy pass, a grid barrier, then block 0
// advances the schedule (depth-first over levels whose output buffer filled)
// and a last barrier publishes it.  Every barrier wait is bounded in time.
struct SchedLevel {                   // per depth, device memory
    unsigned long long n_parents;     // rows of this level (roots at depth 1)
    unsigned long long fresh;         // fresh chunks consumed
    unsigned long long head, tail;    // deferred-chunk ring positions
    unsigned long long parents, lookups, list_words, produced, passes;
};

constexpr unsigned kSchedErrRing = 1u;       // a deferred-chunk ring overflowed
constexpr unsigned kSchedErrPool = 2u;       // a chunk needs more rows than a level buffer holds
constexpr unsigned kSchedErrWait = 4u;       // a grid barrier wait ran out of time
constexpr unsigned kSchedErrLimit = 8u;      // work limit (partial matches produced) reached
constexpr unsigned kSchedErrPasses = 16u;    // more passes than any match can need (a schedule defect)
constexpr unsigned long long kSchedMaxPasses = 1ull << 26;

struct SchedState {
    unsigned int cur;                 // depth of the next pass; 0 = finished
    unsigned int error;               // kSchedErr* bits
    unsigned int bar_count, bar_gen;  // grid barrier
    unsigned int q;                   // levels 1 .. q-1
    unsigned int pad[3];
    unsigned long long passes;
    unsigned long long produced_total;
    unsigned long long work_limit;    // partial matches; 0 = none
    unsigned long long wait_limit_ns; // bound on one barrier wait
    unsigned long long wait_seen_ns;  // longest barrier wait seen
    SchedLevel lv[kMaxQ];
};

// Per-match constants of the persistent engine that ExpandParams does not hold.
struct PersistArgs {
    SchedState* sched;
    uint32_t* levels[kMaxQ];          // level buffer of depth d (rows of d entries), d >= 2
    uint32_t* rings;                  // one deferred ring of ring_cap entries per depth
    uint32_t ring_cap;
    uint64_t n_roots;
    int hold_first_barrier;           // tests: block 0 skips the first barrier
};

// Dynamic shared memory and grid of the persistent kernel for a plan.
size_t persist_smem_bytes(const DevPlan& plan, const uint32_t* nreq_depth, uint32_t stage_words);
// Words of the per-warp membership-list stage (FM_STAGE_WORDS, read once).
uint32_t stage_words_knob();
// Count the last depth from depth q-2 when it has one back edge (FM_PRE_COUNT,
// default 1; 0 launches the last depth as its own level).
bool pre_count_knob();
// One query matched alone on the context's stream (the single-query engine),
// its table (FM_MODE_TABLE) written into `region`, a device buffer of
// `region_rows` rows; used by batches for the queries they match alone.
fm_status match_region(fm_context* ctx, const fm_graph* graph, const fm_query* query, int32_t mode,
                       uint32_t* region, uint64_t region_rows, fm_result* out);
int persist_blocks_per_sm(int last_mode, bool dups, size_t smem);
cudaError_t launch_persist(const ExpandParams& p, const PersistArgs& a, int last_mode, bool dups, int grid,
                           size_t smem, cudaStream_t s);
// Writes the initial schedule (depth 1, n_roots rows) with a one-block kernel.
cudaError_t launch_sched_init(SchedState* S, unsigned q, unsigned long long n_roots, unsigned long long work_limit,
                              unsigned long long wait_ns, cudaStream_t s);

// Launch one level expansion: the main pass, then the heavy-chunk pass
// (fm_match.cu).
cudaError_t launch_expand(const ExpandParams& p, int mode, bool roots, bool dups, int grid, int heavy_grid,
                          int block, size_t smem, cudaStream_t s);
size_t expand_smem_bytes(uint32_t depth, uint32_t nreq, int warps, uint32_t stage_words);
// Let kernel f launch with up to the device's opt-in shared memory (once per
// device; safe from several host threads).
void allow_dynamic_smem(const void* f);
int expand_blocks_per_sm(int mode, bool roots, bool dups, size_t smem, int block);

// The parts of a context other translation units use (fm_host.cu owns it).
struct ContextView {
    bool serving;          // a server owns the slab
    uint32_t bank_rows;    // CurBankSize
    int device, sms;
    cudaStream_t stream;
    char* soln;
    uint64_t soln_bytes;
    uint32_t* output;
    uint64_t output_bytes;
    LaunchCtl* ctl;        // one per depth
    LaunchCtl* h_ctl;      // pinned mirror, one per depth
    uint32_t* defs;
    uint32_t def_cap;
    HeavyEntry* heavy;
    uint32_t heavy_cap;
    SchedState* sched;     // persistent engine schedule (device)
    SchedState* h_sched;   // pinned mirror
};
ContextView context_view(fm_context* c);

// Serving (fm_serve.cpp): per-slot contexts whose regions point into the
// owner's slab.  A view owns its stream, pinned mirrors and events, not its
// memory: `misc` is kContextMiscBytes of device memory (256-byte aligned) for
// its control blocks, deferred lists and heavy entries; the level and table
// regions are set per request.
constexpr uint64_t kContextMiscBytes = 64ull << 20;
fm_status context_create_view(fm_context* owner, char* misc, fm_context** out);
void context_set_regions(fm_context* c, char* soln, uint64_t soln_bytes, uint32_t* output, uint64_t output_bytes);
char* context_slab(fm_context* c, uint64_t* bytes);
bool context_set_serving(fm_context* c, bool on);   // false if already serving
// Batches created by a server are run once: no CUDA-graph capture.
void batch_set_replay(fm_batch* b, bool replay);
// A batch on caller-owned scratch (plans and counts of n queries), so that
// creating and freeing it allocates no device or pinned memory.
struct BatchScratch {
    void* d;
    uint64_t d_bytes;
    void* h;                // pinned
    uint64_t h_bytes;
};
size_t batch_scratch_bytes(uint32_t n, bool device);
fm_status batch_create_scratch(fm_context* ctx, const fm_graph* graph, const fm_query* const* queries, uint32_t n,
                               int32_t mode, const BatchScratch& scratch, fm_batch** out);
// Estimated partial matches per depth under the automatic matching order
// (independent e-lines, label frequencies): the server's footprint model.
void estimate_level_rows(const Plan& P, const DeviceGraph& g, double est[kMaxQ]);

// Device graph build from device edge arrays (fm_graph.cu).
fm_status build_device_graph(DeviceGraph& g, uint32_t V, uint32_t L, uint64_t E, const uint32_t* d_src,
                             const uint32_t* d_dst, const uint32_t* d_lab, cudaStream_t s);

// Host parsers (fm_parse.cpp).
struct EdgeArrays {
    uint32_t V = 0, L = 0;
    std::vector<uint32_t> src, dst, lab;
};
fm_status parse_data_text(const char* text, uint64_t len, EdgeArrays& out);
// The same grammar and checks, parsed on the device straight into a graph
// build (fm_ingest.cu).
fm_status parse_data_text_device(const char* text, uint64_t len, cudaStream_t s, DeviceGraph& g);
fm_status compile_query_text(const char* text, uint64_t len, Plan& out);

}  // namespace fm

struct fm_graph {
    fm::DeviceGraph g;
};

struct fm_query {
    fm::Plan p;
};
