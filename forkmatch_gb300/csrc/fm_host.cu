// fm_host.cu -- C ABI of libforkmatch: contexts, graphs, queries, matching.
//
// The matching driver replaces the reference's host match() (src/smsm.cu:1182-1349)
// and its device-side fork machinery (src/smsm.cu:564-687, 949-1139: CDP child
// launches on bank overflow, tail-launched bank frees).  All levels of a query
// are launched back to back, each reading its parent count from the previous
// level's control block on the device, and the host synchronises once.  If a
// level's buffer filled, the host then walks the levels depth first: it drains
// the deeper levels and relaunches the level on the chunks it deferred or did
// not claim.  Memory is bounded by SOLN_PREALLOC (one buffer per depth) and
// no device code waits on anything.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "fm_internal.h"

namespace fm {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

fm_status cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return FM_ERR_CUDA;
}

}  // namespace fm

using namespace fm;

// ------------------------------------------------------------------ context

struct fm_context {
    fm_knobs knobs{};
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    char* slab = nullptr;
    uint64_t soln_bytes = 0, output_bytes = 0;
    char* soln = nullptr;       // partial-match levels
    uint32_t* output = nullptr; // embedding table
    LaunchCtl* ctl = nullptr;   // device
    MatchTotals* tot = nullptr; // device
    uint32_t* defs = nullptr;   // 2 deferred lists per depth
    uint32_t def_cap = 0;
    HeavyEntry* heavy = nullptr;  // heavy-chunk entries of the current launch
    uint32_t heavy_cap = 0;
    SchedState* sched = nullptr;  // persistent engine schedule (device)
    LaunchCtl* h_ctl = nullptr; // pinned mirrors
    MatchTotals* h_tot = nullptr;
    SchedState* h_sched = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> prof;
    bool serving = false;       // a server owns the slab (fm_match/fm_batch refuse)
};

namespace {

uint64_t env_u64(const char* name, uint64_t dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    char* end = nullptr;
    unsigned long long x = std::strtoull(v, &end, 10);
    return (end && *end == 0) ? (uint64_t)x : dflt;
}

}  // namespace

uint32_t fm::stage_words_knob() {
    // a multiple of 4 words (16-byte bulk copies), at most 4096 words (16 KiB per warp)
    static const uint32_t w = (uint32_t)std::min<uint64_t>(env_u64("FM_STAGE_WORDS", 0), 4096) & ~3u;
    return w;
}

bool fm::pre_count_knob() {
    static const bool on = env_u64("FM_PRE_COUNT", 1) != 0;
    return on;
}

namespace {

// [0, 4 KiB) control blocks, [4 KiB, 8 KiB) match totals and the persistent
// schedule, [8 KiB, 48 MiB) deferred-chunk lists (two per depth, which the
// persistent engine uses as one ring per depth), [48 MiB, 64 MiB) heavy-chunk
// entries
void set_misc(fm_context* c, char* misc) {
    static_assert(kMaxQ * sizeof(LaunchCtl) <= 4096, "per-level control blocks must fit in 4 KiB");
    static_assert(256 + sizeof(SchedState) <= 4096, "totals and schedule must fit in 4 KiB");
    c->ctl = (LaunchCtl*)misc;                 // one control block per depth
    c->tot = (MatchTotals*)(misc + 4096);
    c->sched = (SchedState*)(misc + 4096 + 256);
    c->defs = (uint32_t*)(misc + 8192);
    c->def_cap = (uint32_t)(((48ull << 20) - 8192) / 4 / (2 * kMaxQ));
    c->heavy = (HeavyEntry*)(misc + (48ull << 20));
    c->heavy_cap = (uint32_t)((kContextMiscBytes - (48ull << 20)) / sizeof(HeavyEntry));
}

constexpr uint64_t kMiscBytes = kContextMiscBytes;

}  // namespace

extern "C" {

const char* fm_status_string(fm_status s) {
    switch (s) {
        case FM_OK: return "ok";
        case FM_ERR_ARG: return "invalid argument";
        case FM_ERR_IO: return "file missing or unreadable";
        case FM_ERR_DATA_HEADER0: return "data graph: missing \"t # 0\"";
        case FM_ERR_DATA_TRAILER: return "data graph: missing \"t # -1\"";
        case FM_ERR_DATA_HEADER: return "data graph: malformed header";
        case FM_ERR_DATA_LINE: return "data graph: malformed line";
        case FM_ERR_QUERY_FORMAT: return "query: malformed";
        case FM_ERR_QUERY_MISSING: return "query: missing vertex or edge lines";
        case FM_ERR_DISCONNECTED: return "query: disconnected or not plannable";
        case FM_ERR_UNSUPPORTED: return "unsupported";
        case FM_ERR_POOL: return "SOLN_PREALLOC too small";
        case FM_ERR_OUTPUT_OVERFLOW: return "embedding table truncated at OUTPUT_PREALLOC";
        case FM_ERR_CUDA: return "CUDA error";
        case FM_ERR_DEVICE: return "device status error";
        case FM_ERR_NOMEM: return "out of memory";
        case FM_ERR_LIMIT: return "work limit reached";
    }
    return "unknown";
}

const char* fm_last_error(void) { return g_last_error.c_str(); }

const char* fm_version(void) { return "forkmatch-gb300 0.1 (sm_103a)"; }

int fm_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

void fm_knobs_default(fm_knobs* k) {
    // The reference's defaults (src/environment.cuh:4-6,17) were sized for a
    // 48 GB RTX 8000; GB300 keeps the same proportions with room for a
    // resident graph beside the slab.
    k->prealloc_bytes = env_u64("FM_PREALLOC", 48ull << 30);
    k->soln_prealloc_bytes = env_u64("FM_SOLN_PREALLOC", 24ull << 30);
    k->output_prealloc_bytes = env_u64("FM_OUTPUT_PREALLOC", 18ull << 30);
    k->bank_rows = (uint32_t)env_u64("FM_CUR_BANK_SIZE", 1u << 20);
    k->device = (int32_t)env_u64("FM_DEVICE", 0);
}

void fm_match_opts_default(fm_match_opts* o) {
    std::memset(o, 0, sizeof(*o));
    o->mode = FM_MODE_TABLE;
    o->columns = FM_COLUMNS_REFERENCE;
}

void* fm_host_alloc(uint64_t bytes) {
    void* p = nullptr;
    // mapped + portable: the kernels of any context can write it directly (host_direct)
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void fm_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

void fm_context_destroy(fm_context* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto e : c->prof) cudaEventDestroy(e);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->h_ctl) cudaFreeHost(c->h_ctl);
    if (c->h_tot) cudaFreeHost(c->h_tot);
    if (c->h_sched) cudaFreeHost(c->h_sched);
    if (c->slab) cudaFree(c->slab);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

fm_status fm_context_create(const fm_knobs* knobs, fm_context** out) {
    if (!out) return FM_ERR_ARG;
    *out = nullptr;
    fm_knobs k;
    if (knobs) k = *knobs;
    else fm_knobs_default(&k);
    if (k.bank_rows == 0) k.bank_rows = 1;
    // levels at [0, soln), table at round_up(soln, 256), control blocks at
    // round_down(prealloc - misc, 256): the margin keeps the three disjoint
    uint64_t need = ((k.soln_prealloc_bytes + 255) & ~255ull) + k.output_prealloc_bytes + kMiscBytes + 256;
    if (k.prealloc_bytes < need) {
        set_error("PREALLOC must cover SOLN_PREALLOC + OUTPUT_PREALLOC + 64 MiB");
        return FM_ERR_ARG;
    }
    std::unique_ptr<fm_context, void (*)(fm_context*)> c(new fm_context(), fm_context_destroy);
    c->knobs = k;
    c->device = k.device;
    FM_CUDA(cudaSetDevice(c->device));
    FM_CUDA(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device));
    FM_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    cudaError_t e = cudaMalloc(&c->slab, k.prealloc_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cannot allocate PREALLOC bytes on the device");
        return FM_ERR_NOMEM;
    }
    c->soln_bytes = k.soln_prealloc_bytes;
    c->output_bytes = k.output_prealloc_bytes;
    c->soln = c->slab;
    c->output = (uint32_t*)(c->slab + ((k.soln_prealloc_bytes + 255) & ~255ull));
    // control blocks hold 64-bit atomics: keep them 256-byte aligned whatever PREALLOC is
    set_misc(c.get(), c->slab + ((k.prealloc_bytes - kMiscBytes) & ~255ull));
    FM_CUDA(cudaHostAlloc(&c->h_ctl, kMaxQ * sizeof(LaunchCtl), cudaHostAllocDefault));
    FM_CUDA(cudaHostAlloc(&c->h_tot, sizeof(MatchTotals), cudaHostAllocDefault));
    FM_CUDA(cudaHostAlloc(&c->h_sched, sizeof(SchedState), cudaHostAllocDefault));
    FM_CUDA(cudaEventCreate(&c->ev0));
    FM_CUDA(cudaEventCreate(&c->ev1));
    *out = c.release();
    return FM_OK;
}

void* fm_context_stream(fm_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

// ------------------------------------------------------------------ graphs

static void free_device_graph(DeviceGraph& g) {
    if (g.seg) cudaFree(g.seg);
    if (g.nbr) cudaFree(g.nbr);
    if (g.heads) cudaFree(g.heads);
    if (g.bitmaps) cudaFree(g.bitmaps);
    g.bitmaps = nullptr;
    g.seg = nullptr;
    g.nbr = nullptr;
    g.heads = nullptr;
}

void fm_graph_free(fm_graph* g) {
    if (!g) return;
    cudaSetDevice(g->g.device);
    free_device_graph(g->g);
    delete g;
}

static fm_status graph_from_host_arrays(fm_context* ctx, uint32_t V, uint32_t L, uint64_t E, const uint32_t* src,
                                        const uint32_t* dst, const uint32_t* lab, fm_graph** out) {
    FM_CUDA(cudaSetDevice(ctx->device));
    uint32_t* d = nullptr;
    if (E) {
        cudaError_t e = cudaMalloc(&d, E * 12);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("cannot allocate edge staging buffers");
            return FM_ERR_NOMEM;
        }
        FM_CUDA(cudaMemcpyAsync(d, src, E * 4, cudaMemcpyHostToDevice, ctx->stream));
        FM_CUDA(cudaMemcpyAsync(d + E, dst, E * 4, cudaMemcpyHostToDevice, ctx->stream));
        FM_CUDA(cudaMemcpyAsync(d + 2 * E, lab, E * 4, cudaMemcpyHostToDevice, ctx->stream));
    }
    std::unique_ptr<fm_graph> g(new fm_graph());
    fm_status st = build_device_graph(g->g, V, L, E, d, d + E, d + 2 * E, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (d) cudaFree(d);
    if (st != FM_OK) {
        free_device_graph(g->g);
        return st;
    }
    g->g.label_count.assign(L, 0);   // label frequencies for the matching-order cost model
    for (uint64_t i = 0; i < E; i++) g->g.label_count[lab[i]]++;
    *out = g.release();
    return FM_OK;
}

fm_status fm_graph_from_edges(fm_context* ctx, uint32_t vertices, uint32_t label_slots, uint64_t edges,
                              const uint32_t* src, const uint32_t* dst, const uint32_t* label, fm_graph** out) {
    if (!ctx || !out || (edges && (!src || !dst || !label))) return FM_ERR_ARG;
    *out = nullptr;
    if (label_slots > FM_MAX_LABEL + 1) {
        set_error("label_slots above 256 (query labels are 8-bit)");
        return FM_ERR_UNSUPPORTED;
    }
    return graph_from_host_arrays(ctx, vertices, label_slots, edges, src, dst, label, out);
}

fm_status fm_graph_load_text(fm_context* ctx, const char* text, uint64_t len, fm_graph** out) {
    if (!ctx || !out || (!text && len)) return FM_ERR_ARG;
    *out = nullptr;
    FM_CUDA(cudaSetDevice(ctx->device));
    std::unique_ptr<fm_graph> g(new fm_graph());
    fm_status st = parse_data_text_device(text, len, ctx->stream, g->g);
    if (st != FM_OK) {
        free_device_graph(g->g);
        return st;
    }
    *out = g.release();
    return FM_OK;
}

static bool read_file(const char* path, std::string& buf) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    f.seekg(0, std::ios::end);
    std::streamoff n = f.tellg();
    if (n < 0) return false;
    f.seekg(0, std::ios::beg);
    buf.resize((size_t)n);
    if (n && !f.read(&buf[0], n)) return false;
    return true;
}

// Binary graph cache: the parsed e-lines of a .g file, so a large graph is
// loaded without parsing text again.  Little-endian:
//   "FMGB0001", u32 vertices, u32 label slots, u64 e-lines, u32 label bytes
//   (1), u32 0, then src[E] u32, dst[E] u32, label[E] u8.
namespace {
const char kCacheMagic[8] = {'F', 'M', 'G', 'B', '0', '0', '0', '1'};
struct CacheHeader {
    char magic[8];
    uint32_t V, L;
    uint64_t E;
    uint32_t lab_bytes, reserved;
};
static_assert(sizeof(CacheHeader) == 32, "cache header layout");
}  // namespace

fm_status fm_graph_write_cache(const char* text_path, const char* cache_path) {
    if (!text_path || !cache_path) return FM_ERR_ARG;
    std::string buf;
    if (!read_file(text_path, buf)) {
        set_error(std::string("missing file ") + text_path);
        return FM_ERR_IO;
    }
    EdgeArrays ea;
    fm_status st = parse_data_text(buf.data(), buf.size(), ea);
    if (st != FM_OK) return st;
    std::string().swap(buf);
    CacheHeader h;
    std::memcpy(h.magic, kCacheMagic, 8);
    h.V = ea.V;
    h.L = ea.L;
    h.E = ea.src.size();
    h.lab_bytes = 1;
    h.reserved = 0;
    std::vector<uint8_t> lab8(h.E);
    for (uint64_t i = 0; i < h.E; i++) lab8[i] = (uint8_t)ea.lab[i];   // label slots <= 256
    std::ofstream f(cache_path, std::ios::binary | std::ios::trunc);
    if (!f) {
        set_error(std::string("cannot write ") + cache_path);
        return FM_ERR_IO;
    }
    f.write((const char*)&h, sizeof(h));
    f.write((const char*)ea.src.data(), h.E * 4);
    f.write((const char*)ea.dst.data(), h.E * 4);
    f.write((const char*)lab8.data(), h.E);
    if (!f) {
        set_error(std::string("cannot write ") + cache_path);
        return FM_ERR_IO;
    }
    return FM_OK;
}

fm_status fm_graph_load_file(fm_context* ctx, const char* path, fm_graph** out) {
    if (!ctx || !path || !out) return FM_ERR_ARG;
    *out = nullptr;
    std::string buf;
    if (!read_file(path, buf)) {
        set_error(std::string("missing file ") + path);
        return FM_ERR_IO;
    }
    if (buf.size() >= sizeof(CacheHeader) && std::memcmp(buf.data(), kCacheMagic, 8) == 0) {
        CacheHeader h;
        std::memcpy(&h, buf.data(), sizeof(h));
        if (h.lab_bytes != 1 || h.L == 0 || h.L > FM_MAX_LABEL + 1 ||
            buf.size() != sizeof(h) + h.E * 9) {
            set_error("graph cache: bad header or size");
            return FM_ERR_DATA_HEADER;
        }
        const char* p = buf.data() + sizeof(h);
        std::vector<uint32_t> src(h.E), dst(h.E), lab(h.E);
        std::memcpy(src.data(), p, h.E * 4);
        std::memcpy(dst.data(), p + h.E * 4, h.E * 4);
        const uint8_t* l8 = (const uint8_t*)(p + h.E * 8);
        for (uint64_t i = 0; i < h.E; i++) lab[i] = l8[i];
        std::string().swap(buf);
        return graph_from_host_arrays(ctx, h.V, h.L, h.E, src.data(), dst.data(), lab.data(), out);
    }
    return fm_graph_load_text(ctx, buf.data(), buf.size(), out);
}

fm_status fm_graph_get_info(const fm_graph* g, fm_graph_info* info) {
    if (!g || !info) return FM_ERR_ARG;
    const DeviceGraph& d = g->g;
    info->vertices = d.V;
    info->label_slots = d.L;
    info->edges = d.E;
    info->segments = d.segments;
    info->long_segments = d.long_segments;
    info->nbr_words = d.nbr_words;
    info->max_list = d.max_len;
    info->has_duplicates = d.has_dups;
    info->bitmaps = d.n_bitmaps;
    info->bitmap_min_len = d.bm_min_len;
    info->bitmap_bytes = (uint64_t)d.n_bitmaps * d.bm_words * 4;
    info->device_bytes = (uint64_t)d.L * d.V * 16 + d.nbr_words * 4 + d.segments * 4 + info->bitmap_bytes;
    info->build_ms = d.build_ms;
    return FM_OK;
}

// ------------------------------------------------------------------ queries

fm_status fm_query_compile_text(const char* text, uint64_t len, fm_query** out) {
    if (!out || (!text && len)) return FM_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<fm_query> q(new fm_query());
    fm_status st = compile_query_text(text, len, q->p);
    if (st != FM_OK) return st;
    *out = q.release();
    return FM_OK;
}

fm_status fm_query_compile_file(const char* path, fm_query** out) {
    if (!path || !out) return FM_ERR_ARG;
    *out = nullptr;
    std::string buf;
    if (!read_file(path, buf)) {
        set_error(std::string("missing file ") + path);
        return FM_ERR_IO;
    }
    return fm_query_compile_text(buf.data(), buf.size(), out);
}

fm_status fm_query_get_info(const fm_query* q, fm_query_info* info) {
    if (!q || !info) return FM_ERR_ARG;
    std::memset(info, 0, sizeof(*info));
    const Plan& p = q->p;
    info->q = p.q;
    info->e_lines = p.e_lines;
    info->max_valency = p.max_valency;
    for (uint32_t d = 0; d < p.q; d++) {
        info->order[d] = p.inv[p.order_local[d]];
        info->local_of_depth[d] = p.order_local[d];
        info->inv[d] = p.inv[d];
        info->nreq[d] = p.nreq[d];
        info->pk_dist[d] = p.pk_dist[d];
        for (uint32_t i = 0; i < p.nreq[d]; i++) {
            info->req_climb[d][i] = p.req_climb[d][i];
            info->req_label[d][i] = p.req_label[d][i];
            info->req_refl[d][i] = p.req_refl[d][i];
        }
    }
    info->automorphisms = p.automorphisms;
    return FM_OK;
}

void fm_query_free(fm_query* q) { delete q; }

}  // extern "C"

// ------------------------------------------------------------------ matching

namespace {

struct MatchRun {
    fm_context* ctx;
    const DeviceGraph* g;
    const Plan* plan;
    const uint32_t* nreq_depth = nullptr;   // requirements per depth of the order in use
    ExpandParams base;
    cudaStream_t s;
    bool table;
    bool dups;
    uint64_t level_cap;              // rows per level buffer
    uint32_t* level[kMaxQ];          // SoA buffers, rows with d entries at level[d]
    fm_result* res;
    bool profile;
    size_t prof_used = 0;
    int block = 256;
    uint64_t work_limit = 0;         // partial matches produced, checked between launches
    // count mode with one back edge at the last depth: depth q-2 counts its
    // survivors' extensions (ExpandParams::pre_count) and depth q-1 is never
    // launched
    bool pre = false;

    uint32_t last_depth() const { return plan->q - 1 - (pre ? 1u : 0u); }

    bool over_limit() const {
        if (!work_limit) return false;
        uint64_t s = 0;
        for (uint32_t d = 1; d + 1 < plan->q; d++) s += res->level[d].produced;
        return s > work_limit;
    }

    int mode_of(uint32_t d) const {
        return (d == last_depth()) ? (table ? kModeLastTable : kModeLastCount) : kModeMid;
    }

    // Pre-count: the last depth's work counters, which the counting level
    // added to the last depth's control block, and the counting level's
    // survivors (its "produced" rows, never stored).
    fm_status finish_pre() {
        if (!pre) return FM_OK;
        const uint32_t q = plan->q;
        FM_CUDA(cudaMemcpyAsync(ctx->h_ctl + q - 1, ctx->ctl + q - 1, sizeof(LaunchCtl), cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        const LaunchCtl& c = ctx->h_ctl[q - 1];
        fm_level_stats& ls = res->level[q - 1];
        ls.parents = c.parents;
        ls.lookups = c.lookups;
        ls.list_words = c.list_words;
        res->level[q - 2].produced = c.parents;
        return FM_OK;
    }
    uint32_t* def_list(uint32_t d, int which) const {
        return ctx->defs + (size_t)(2 * d + which) * ctx->def_cap;
    }
    fm_status begin_timing(cudaEvent_t& e0, cudaEvent_t& e1) {
        while (ctx->prof.size() < prof_used + 2) {
            cudaEvent_t e;
            FM_CUDA(cudaEventCreate(&e));
            ctx->prof.push_back(e);
        }
        e0 = ctx->prof[prof_used++];
        e1 = ctx->prof[prof_used++];
        FM_CUDA(cudaEventRecord(e0, s));
        return FM_OK;
    }
    void add_stats(uint32_t d, const LaunchCtl& c) {
        fm_level_stats& ls = res->level[d];
        ls.launches++;
        res->launches++;
        res->passes++;
        ls.parents += c.parents;
        ls.lookups += c.lookups;
        ls.list_words += c.list_words;
        if (mode_of(d) == kModeMid) ls.produced += c.produced;
    }

    // Optimistic pass: every level launched back to back, level d reading its
    // parent count from level d-1's control block on the device; one sync.
    // Levels whose buffer filled (deferred or unclaimed chunks) are then
    // resumed deepest first, so a level never writes into a buffer that a
    // deeper level still has to read.
    fm_status run(uint64_t n_roots) {
        const uint32_t q = plan->q;
        const uint32_t last = last_depth();
        cudaEvent_t ev[kMaxQ][2] = {};
        if (pre) FM_CUDA(cudaMemsetAsync(ctx->ctl + q - 1, 0, sizeof(LaunchCtl), s));
        for (uint32_t d = 1; d <= last; d++) {
            const int mode = mode_of(d);
            const bool roots = d == 1;
            const size_t smem = expand_smem_bytes(d, nreq_depth[d], block / 32,
                                                  nreq_depth[d] >= 2 ? base.stage_words : 0);
            const int per_sm = expand_blocks_per_sm(mode, roots, dups, smem, block);
            const int full = ctx->sms * per_sm;
            ExpandParams p = base;
            p.pin = roots ? nullptr : level[d];
            p.pstride = level_cap;
            p.depth = d;
            p.def_in = def_list(d, 0);
            p.ndef_in = 0;
            p.fresh_base = 0;
            p.def_out = def_list(d, 1);
            p.def_cap = ctx->def_cap;
            p.pout = (mode == kModeMid) ? level[d + 1] : nullptr;
            p.ocap = level_cap;
            p.ctl = ctx->ctl + d;
            int grid = full;
            if (roots) {
                p.n_parents = n_roots;
                p.n_items = (n_roots + 31) / 32;
                grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((p.n_items + 7) / 8, (uint64_t)full));
            } else {
                p.n_parents_dev = &ctx->ctl[d - 1].produced;
            }
            FM_CUDA(cudaMemsetAsync(ctx->ctl + d, 0, sizeof(LaunchCtl), s));
            if (profile) FM_TRY(begin_timing(ev[d][0], ev[d][1]));
            FM_CUDA(launch_expand(p, mode, roots, dups, grid, full, block, smem, s));
            if (profile) FM_CUDA(cudaEventRecord(ev[d][1], s));
        }
        FM_CUDA(cudaMemcpyAsync(ctx->h_ctl, ctx->ctl, q * sizeof(LaunchCtl), cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        uint64_t n_parents[kMaxQ] = {};
        for (uint32_t d = 1; d <= last; d++) {
            const LaunchCtl& c = ctx->h_ctl[d];
            n_parents[d] = d == 1 ? n_roots : ctx->h_ctl[d - 1].produced;
            add_stats(d, c);
            if (profile) {
                float ms = 0;
                cudaEventElapsedTime(&ms, ev[d][0], ev[d][1]);
                res->level[d].kernel_ms += ms;
            }
            if (c.error) {
                set_error((c.error & 2u) ? "a list stage's bounded wait ran out" : "deferred-chunk list overflow");
                return FM_ERR_DEVICE;
            }
        }
        if (over_limit()) return FM_ERR_LIMIT;
        LaunchCtl snap[kMaxQ];
        std::memcpy(snap, ctx->h_ctl, q * sizeof(LaunchCtl));
        for (uint32_t d = last; d >= 1; d--) {
            if (mode_of(d) != kModeMid) continue;   // the last level never defers
            const LaunchCtl& c = snap[d];
            const uint64_t items = (n_parents[d] + 31) / 32;
            const uint64_t claimed = std::min<uint64_t>(c.claim, items);
            if (c.ndef == 0 && claimed == items) continue;
            // every chunk claimed in the optimistic pass was fresh and was either
            // processed or deferred (its id is in the pass's def_out list)
            fm_status st = drain_level(d, n_parents[d], d == 1, c.ndef, claimed, def_list(d, 1), def_list(d, 0));
            if (st != FM_OK) return st;
        }
        return finish_pre();
    }

    // Persistent engine: one cooperative launch runs every pass; the device
    // schedules them (depth first over levels whose buffer filled) from the
    // per-depth work queues.  Returns FM_ERR_UNSUPPORTED (nothing launched)
    // when no block of the kernel fits an SM with this plan's shared memory.
    fm_status run_persistent(uint64_t n_roots, const fm_match_opts& opts) {
        const uint32_t q = plan->q;
        const int last_mode = table ? kModeLastTable : kModeLastCount;
        const size_t smem = persist_smem_bytes(base.plan, nreq_depth, base.stage_words);
        const int per_sm = persist_blocks_per_sm(last_mode, dups, smem);
        if (per_sm < 1) return FM_ERR_UNSUPPORTED;
        const int grid = ctx->sms * per_sm;
        SchedState& h = *ctx->h_sched;
        const unsigned long long wait_ns =
            (unsigned long long)(opts.wait_limit_ms ? opts.wait_limit_ms : 60000u) * 1000000ull;
        FM_CUDA(launch_sched_init(ctx->sched, q, n_roots, work_limit, wait_ns, s));
        FM_CUDA(cudaMemsetAsync(ctx->ctl, 0, q * sizeof(LaunchCtl), s));
        PersistArgs a;
        std::memset(&a, 0, sizeof(a));
        a.sched = ctx->sched;
        for (uint32_t d = 0; d < (uint32_t)kMaxQ; d++) a.levels[d] = level[d];
        a.rings = ctx->defs;
        a.ring_cap = 2 * ctx->def_cap;
        a.n_roots = n_roots;
        a.hold_first_barrier = opts.test_stall_barrier ? 1 : 0;
        ExpandParams p = base;
        p.pstride = level_cap;
        p.ocap = level_cap;
        p.ctl = ctx->ctl;
        FM_CUDA(launch_persist(p, a, last_mode, dups, grid, smem, s));
        FM_CUDA(cudaMemcpyAsync(&h, ctx->sched, sizeof(h), cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        for (uint32_t d = 1; d < q; d++) {
            fm_level_stats& ls = res->level[d];
            ls.parents += h.lv[d].parents;
            ls.lookups += h.lv[d].lookups;
            ls.list_words += h.lv[d].list_words;
            ls.produced += h.lv[d].produced;
            ls.launches += (uint32_t)h.lv[d].passes;
        }
        res->launches += 1;
        res->passes += (uint32_t)h.passes;
        res->max_wait_ns = h.wait_seen_ns;
        if (h.error & kSchedErrWait) {
            set_error("a bounded wait of the persistent kernel ran out (a grid barrier after wait_limit_ms, or a list stage)");
            return FM_ERR_DEVICE;
        }
        if (h.error & kSchedErrPasses) {
            set_error("the persistent schedule exceeded its pass bound");
            return FM_ERR_DEVICE;
        }
        if (h.error & kSchedErrRing) {
            set_error("deferred-chunk ring overflow");
            return FM_ERR_DEVICE;
        }
        if (h.error & kSchedErrPool) {
            set_error("one 32-parent chunk needs more rows than a level buffer holds; raise SOLN_PREALLOC");
            return FM_ERR_POOL;
        }
        if (h.error & kSchedErrLimit) return FM_ERR_LIMIT;
        return finish_pre();
    }

    // Host-driven depth-first loop for one level (used when a level's buffer
    // filled): relaunch on deferred + unclaimed chunks, draining deeper levels
    // after every launch.  `fresh` counts fresh chunks already processed or
    // deferred; `def_a` holds `ndef_in` deferred chunk ids.
    fm_status drain_level(uint32_t d, uint64_t n_parents, bool roots, uint32_t ndef_in, uint64_t fresh,
                          uint32_t* def_a, uint32_t* def_b) {
        const uint32_t q = plan->q;
        const int mode = mode_of(d);
        const uint64_t n_chunks = (n_parents + 31) / 32;
        const size_t smem =
            expand_smem_bytes(d, nreq_depth[d], block / 32, nreq_depth[d] >= 2 ? base.stage_words : 0);
        const int per_sm = expand_blocks_per_sm(mode, roots, dups, smem, block);
        (void)q;
        while (true) {
            const uint64_t items = ndef_in + (n_chunks - fresh);
            if (items == 0) break;
            ExpandParams p = base;
            p.pin = roots ? nullptr : level[d];
            p.pstride = level_cap;
            p.n_parents = n_parents;
            p.depth = d;
            p.def_in = def_a;
            p.ndef_in = ndef_in;
            p.fresh_base = fresh;
            p.n_items = items;
            p.def_out = def_b;
            p.def_cap = ctx->def_cap;
            p.pout = (mode == kModeMid) ? level[d + 1] : nullptr;
            p.ocap = level_cap;
            p.ctl = ctx->ctl + d;
            uint64_t want = (items + (block / 32) - 1) / (block / 32);
            int grid = (int)std::min<uint64_t>(want, (uint64_t)ctx->sms * per_sm);
            if (grid < 1) grid = 1;
            FM_CUDA(cudaMemsetAsync(ctx->ctl + d, 0, sizeof(LaunchCtl), s));
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (profile) FM_TRY(begin_timing(e0, e1));
            FM_CUDA(launch_expand(p, mode, roots, dups, grid, ctx->sms * per_sm, block, smem, s));
            if (profile) FM_CUDA(cudaEventRecord(e1, s));
            FM_CUDA(cudaMemcpyAsync(ctx->h_ctl + d, ctx->ctl + d, sizeof(LaunchCtl), cudaMemcpyDeviceToHost, s));
            FM_CUDA(cudaStreamSynchronize(s));
            const LaunchCtl c = ctx->h_ctl[d];
            if (profile) {
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                res->level[d].kernel_ms += ms;
            }
            add_stats(d, c);
            if (c.error) {
                set_error((c.error & 2u) ? "a list stage's bounded wait ran out" : "deferred-chunk list overflow");
                return FM_ERR_DEVICE;
            }
            if (over_limit()) return FM_ERR_LIMIT;
            const uint64_t claimed = std::min<uint64_t>(c.claim, items);
            const uint64_t fresh_claimed = claimed > ndef_in ? claimed - ndef_in : 0;
            const uint64_t carry = ndef_in > claimed ? ndef_in - claimed : 0;
            fresh += fresh_claimed;
            uint64_t ndef_out = c.ndef;
            if (ndef_out + carry > ctx->def_cap) {
                set_error("deferred-chunk list overflow");
                return FM_ERR_DEVICE;
            }
            if (carry) {
                FM_CUDA(cudaMemcpyAsync(def_b + ndef_out, def_a + claimed, carry * 4, cudaMemcpyDeviceToDevice, s));
                ndef_out += carry;
            }
            if (mode == kModeMid) {
                const uint64_t done_chunks = claimed - c.ndef;
                if (done_chunks == 0 && c.produced == 0 && ndef_out == items) {
                    set_error("one 32-parent chunk needs more rows than a level buffer holds; raise SOLN_PREALLOC");
                    return FM_ERR_POOL;
                }
                if (c.produced) {
                    fm_status st = drain_level(d + 1, c.produced, false, 0, 0, def_list(d + 1, 0), def_list(d + 1, 1));
                    if (st != FM_OK) return st;
                }
            }
            std::swap(def_a, def_b);
            ndef_in = (uint32_t)ndef_out;
        }
        return FM_OK;
    }
};

__global__ void k_iota_rows(uint32_t* out, uint64_t n, uint32_t first, uint64_t cap) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n && i < cap; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = first + (uint32_t)i;
}

}  // namespace

namespace {

// fm_match with the table written into `region` (device memory, `region_rows`
// rows) instead of the start of OUTPUT_PREALLOC when `region` is set.
fm_status match_impl(fm_context* ctx, const fm_graph* graph, const fm_query* query, const fm_match_opts& opts,
                     fm_result* out, uint32_t* region, uint64_t region_rows) {
    std::memset(out, 0, sizeof(*out));
    const DeviceGraph& g = graph->g;
    const Plan& pl = query->p;
    if (ctx->serving) {
        set_error("the context's slab belongs to a server (fm_server_create)");
        return FM_ERR_ARG;
    }
    if (g.device != ctx->device) {
        set_error("graph and context live on different devices");
        return FM_ERR_ARG;
    }
    FM_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = opts.stream ? (cudaStream_t)opts.stream : ctx->stream;
    const uint32_t q = pl.q;
    out->q = q;
    uint32_t rb = opts.root_begin, re = opts.root_end ? opts.root_end : g.V;
    if (re > g.V) re = g.V;
    if (rb > re) rb = re;
    const bool table = opts.mode == FM_MODE_TABLE;
    // The table lives in the context's OUTPUT_PREALLOC region, or -- host_direct --
    // in the caller's pinned host buffer, written by the kernels over the host link.
    const bool direct = table && opts.host_direct && opts.host_rows;
    uint32_t* table_ptr = region ? region : ctx->output;
    uint64_t table_cap = region ? region_rows : ctx->output_bytes / (4ull * q);
    if (direct) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, opts.host_rows) != cudaSuccess || a.type != cudaMemoryTypeHost ||
            !a.devicePointer) {
            cudaGetLastError();
            set_error("host_direct needs host_rows in pinned host memory (fm_host_alloc)");
            return FM_ERR_ARG;
        }
        table_ptr = (uint32_t*)a.devicePointer;
        table_cap = opts.host_rows_cap;
    }

    // matching order: the reference's, or the cheapest one for this graph
    uint32_t order[kMaxQ];
    uint32_t nreq[kMaxQ], climb[kMaxQ][kMaxQ], rlab[kMaxQ][kMaxQ];
    // With duplicate e-lines the reference's multiplicity is a per-depth
    // minimum over the intersected lists (src/smsm.cu:73-140), which depends on
    // which back edges share a depth: only its own order reproduces its count.
    bool use_ref = opts.order == FM_ORDER_REFERENCE || g.has_dups;
    if (!use_ref) {
        choose_order(pl, g, order);
        if (!order_requirements(pl, order, nreq, climb, rlab)) use_ref = true;
    }
    if (use_ref) {
        for (uint32_t d = 0; d < q; d++) {
            order[d] = pl.order_local[d];
            nreq[d] = pl.nreq[d];
            for (uint32_t i = 0; i < pl.nreq[d]; i++) {
                climb[d][i] = pl.req_climb[d][i];
                rlab[d][i] = pl.req_label[d][i];
            }
        }
    }
    uint32_t ref_depth[kMaxQ];   // reference depth of each local vertex: fixes the table layout
    for (uint32_t d = 0; d < q; d++) ref_depth[pl.order_local[d]] = d;

    // device plan
    MatchRun run;
    std::memset(&run.base, 0, sizeof(run.base));
    DevPlan& dp = run.base.plan;
    dp.q = q;
    uint32_t r = 0;
    bool impossible = false;
    for (uint32_t d = 0; d < q; d++) {
        dp.nreq[d] = nreq[d];
        dp.req_begin[d] = r;
        for (uint32_t i = 0; i < nreq[d]; i++, r++) {
            dp.req_anc[r] = (uint8_t)(d - climb[d][i]);
            dp.req_label[r] = (uint8_t)rlab[d][i];
            if (rlab[d][i] >= g.L) impossible = true;   // label absent from the data graph
        }
        const uint32_t v = order[d];
        dp.out_col[d] = (uint8_t)(opts.columns == FM_COLUMNS_QUERY_ID ? pl.inv[v] : q - 1 - ref_depth[v]);
        dp.col_depth[dp.out_col[d]] = (uint8_t)d;
    }
    run.nreq_depth = nreq;
    if ((uint64_t)g.max_len * 32 >= (1ull << 32)) {
        set_error("a neighbour list is longer than 2^27");
        return FM_ERR_UNSUPPORTED;
    }

    FM_CUDA(cudaMemsetAsync(ctx->tot, 0, sizeof(MatchTotals), s));
    FM_CUDA(cudaEventRecord(ctx->ev0, s));
    bool limited = false;
    if (q == 1) {
        uint64_t n = re - rb;
        if (table && n) {
            k_iota_rows<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(table_ptr, n, rb, table_cap);
            FM_CUDA(cudaGetLastError());
        }
        out->count = n;
    } else if (!impossible && re > rb) {
        // pre-count: the last depth is counted from depth q-2, so it needs no
        // level buffer (graphs with duplicate e-lines enumerate it)
        run.pre = !table && !g.has_dups && q >= 3 && nreq[q - 1] == 1 && pre_count_knob();
        const uint32_t stored = q - (run.pre ? 1u : 0u);   // depths with a level buffer: 2 .. stored-1
        uint64_t sum_cols = 0;
        for (uint32_t d = 2; d < stored; d++) sum_cols += d;
        uint64_t cap = sum_cols ? ctx->soln_bytes / (4ull * sum_cols) : 0;
        const uint64_t bank = ctx->knobs.bank_rows;
        if (sum_cols) {
            cap = std::min<uint64_t>(cap, 0xffffffffull - 64);   // parent indices are 32-bit
            cap = cap / bank * bank;
            if (cap < (uint64_t)g.max_len * 32 + 32 || cap == 0) {
                set_error("SOLN_PREALLOC cannot hold one 32-parent chunk per level for this graph");
                return FM_ERR_POOL;
            }
        }
        run.ctx = ctx;
        run.g = &g;
        run.plan = &pl;
        run.s = s;
        run.table = table;
        run.dups = g.has_dups != 0;
        run.level_cap = cap;
        run.res = out;
        run.profile = opts.profile != 0;
        uint64_t off = 0;
        for (uint32_t d = 0; d < kMaxQ; d++) run.level[d] = nullptr;
        for (uint32_t d = 2; d < stored; d++) {
            run.level[d] = (uint32_t*)(ctx->soln + off);
            off += 4ull * d * cap;
        }
        ExpandParams& b = run.base;
        b.seg = g.seg;
        b.nbr = g.nbr;
        b.bm = g.bitmaps;
        b.bm_words = g.bm_words;
        b.V = g.V;
        b.root_begin = rb;
        // Over the full vertex range the roots are the vertices that have an
        // e-line of a depth-1 label (the shortest such list): any other root
        // fails its depth-1 lookup.  A partial range walks the range itself.
        uint64_t n_roots = re - rb;
        b.root_list = nullptr;
        if (rb == 0 && re == g.V && !g.head_off.empty()) {
            for (uint32_t i = 0; i < nreq[1]; i++) {
                const uint32_t l = dp.req_label[dp.req_begin[1] + i];
                const uint64_t n = g.head_off[l + 1] - g.head_off[l];
                if (!b.root_list || n < n_roots) {
                    b.root_list = g.heads + g.head_off[l];
                    n_roots = n;
                }
            }
        }
        b.table = table_ptr;
        b.table_cap = table_cap;
        b.table_vec4 = (q % 4 == 0 && ((uintptr_t)table_ptr % 16) == 0) ? 1u : 0u;
        b.ctl = ctx->ctl;
        b.tot = ctx->tot;
        b.heavy = ctx->heavy;
        b.heavy_cap = ctx->heavy_cap;
        b.work_limit = opts.work_limit;
        b.stage_words = stage_words_knob();
        b.pre_count = run.pre ? 1u : 0u;
        b.self_loops = g.has_self_loops ? 1u : 0u;
        out->pre_counted = run.pre ? 1 : 0;
        run.work_limit = opts.work_limit;
        fm_status st = FM_ERR_UNSUPPORTED;
        out->engine = FM_ENGINE_LEVELS;
        if (opts.engine == FM_ENGINE_PERSISTENT && !opts.profile) {
            st = run.run_persistent(n_roots, opts);
            if (st != FM_ERR_UNSUPPORTED) out->engine = FM_ENGINE_PERSISTENT;
        }
        if (st == FM_ERR_UNSUPPORTED) st = run.run(n_roots);
        if (st == FM_ERR_LIMIT) limited = true;
        else if (st != FM_OK) return st;
    }
    FM_CUDA(cudaEventRecord(ctx->ev1, s));
    FM_CUDA(cudaMemcpyAsync(ctx->h_tot, ctx->tot, sizeof(MatchTotals), cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    out->device_ms = ms;
    if (q > 1) out->count = table ? ctx->h_tot->table_pos : ctx->h_tot->count;
    out->rows = table ? std::min<uint64_t>(out->count, table_cap) : 0;
    out->truncated = table && out->count > table_cap;
    out->rows_device = (table && !direct) ? table_ptr : nullptr;
    if (q > 1) out->level[q - 1].produced = out->count;
    if (direct) {
        out->rows_copied = out->rows;   // already in host memory
    } else if (table && opts.host_rows && out->rows) {
        uint64_t n = std::min<uint64_t>(out->rows, opts.host_rows_cap);
        FM_CUDA(cudaMemcpyAsync(opts.host_rows, table_ptr, n * q * 4, cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        out->rows_copied = n;
    }
    out->h2d_bytes = out->launches * sizeof(ExpandParams);
    out->d2h_bytes = out->launches * sizeof(LaunchCtl) + sizeof(MatchTotals) + out->rows_copied * q * 4;
    if (limited || (ctx->h_tot->error & kLimitFlag)) {
        set_error("work limit reached; count and rows are a lower bound");
        return FM_ERR_LIMIT;
    }
    if (out->truncated) {
        set_error("embedding table truncated at OUTPUT_PREALLOC; count is exact");
        return FM_ERR_OUTPUT_OVERFLOW;
    }
    return FM_OK;
}

}  // namespace

extern "C" fm_status fm_match(fm_context* ctx, const fm_graph* graph, const fm_query* query,
                              const fm_match_opts* opts_in, fm_result* out) {
    if (!ctx || !graph || !query || !out) return FM_ERR_ARG;
    fm_match_opts opts;
    if (opts_in) opts = *opts_in;
    else fm_match_opts_default(&opts);
    return match_impl(ctx, graph, query, opts, out, nullptr, 0);
}

fm_status fm::match_region(fm_context* ctx, const fm_graph* graph, const fm_query* query, int32_t mode,
                           uint32_t* region, uint64_t region_rows, fm_result* out) {
    fm_match_opts opts;
    fm_match_opts_default(&opts);
    opts.mode = mode;
    return match_impl(ctx, graph, query, opts, out, mode == FM_MODE_TABLE ? region : nullptr, region_rows);
}

fm_status fm::context_create_view(fm_context* owner, char* misc, fm_context** out) {
    *out = nullptr;
    std::unique_ptr<fm_context, void (*)(fm_context*)> c(new fm_context(), fm_context_destroy);
    c->knobs = owner->knobs;
    c->device = owner->device;
    c->sms = owner->sms;
    FM_CUDA(cudaSetDevice(c->device));
    FM_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    set_misc(c.get(), misc);
    FM_CUDA(cudaHostAlloc(&c->h_ctl, kMaxQ * sizeof(LaunchCtl), cudaHostAllocDefault));
    FM_CUDA(cudaHostAlloc(&c->h_tot, sizeof(MatchTotals), cudaHostAllocDefault));
    FM_CUDA(cudaHostAlloc(&c->h_sched, sizeof(SchedState), cudaHostAllocDefault));
    FM_CUDA(cudaEventCreate(&c->ev0));
    FM_CUDA(cudaEventCreate(&c->ev1));
    *out = c.release();
    return FM_OK;
}

void fm::context_set_regions(fm_context* c, char* soln, uint64_t soln_bytes, uint32_t* output, uint64_t output_bytes) {
    c->soln = soln;
    c->soln_bytes = soln_bytes;
    c->output = output;
    c->output_bytes = output_bytes;
}

char* fm::context_slab(fm_context* c, uint64_t* bytes) {
    *bytes = c->knobs.prealloc_bytes;
    return c->slab;
}

bool fm::context_set_serving(fm_context* c, bool on) {
    if (on && c->serving) return false;
    c->serving = on;
    return true;
}

fm::ContextView fm::context_view(fm_context* c) {
    ContextView v;
    v.serving = c->serving;
    v.bank_rows = c->knobs.bank_rows;
    v.device = c->device;
    v.sms = c->sms;
    v.stream = c->stream;
    v.soln = c->soln;
    v.soln_bytes = c->soln_bytes;
    v.output = c->output;
    v.output_bytes = c->output_bytes;
    v.ctl = c->ctl;
    v.h_ctl = c->h_ctl;
    v.defs = c->defs;
    v.def_cap = c->def_cap;
    v.heavy = c->heavy;
    v.heavy_cap = c->heavy_cap;
    v.sched = c->sched;
    v.h_sched = c->h_sched;
    return v;
}
