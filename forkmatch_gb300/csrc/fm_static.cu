// fm_static.cu -- fm_match_static: matching that allocates nothing.
//
// Some callers cannot call cudaMalloc at match time: a host application that
// owns all device memory through its own pool and forbids allocations it did
// not make, or a latency-critical serving loop where an allocation (and the
// device synchronisation cudaMalloc/cudaFree can imply) is not acceptable.
// fm_match_static gives them the matcher with every piece of scratch memory
// (level buffers, control blocks, work lists) taken from one fixed array in
// this library's device data, so the call allocates no memory anywhere.  The
// caller still provides the inputs (a resident graph, a compiled query) and
// the outputs (the count, and optionally a device buffer for the table).
//
// The array is shared by every call on a device and keeps the previous call's
// contents; the parts that must start at zero are cleared by each call.
// Calls that overlap on the GPU (two streams, or two host threads) race on it,
// so callers must serialise them.  Its size is fixed at kStaticScratchBytes;
// a graph/query pair whose levels do not fit is rejected with FM_ERR_POOL.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "fm_internal.h"

namespace fm {
namespace {

constexpr uint64_t kStaticScratchBytes = 64ull << 20;   // the fixed maximum
constexpr uint64_t kStaticCtlBytes = 4096;
constexpr uint32_t kStaticDefCap = 32768;                // entries per deferred list (two per depth)
constexpr uint32_t kStaticHeavyCap = 65536;              // heavy-chunk entries

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch per device, looked up once with the
// device current (the host-side symbol is not a device address).
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

fm_status scratch_for_device(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal out of range for the static scratch table");
        return FM_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = (unsigned char*)g_scratch_addr[dev];
    return FM_OK;
}

// Makes a device current for the scope of one call and restores the
// caller's current device when the scope ends.
struct DeviceGuard {
    int prev = -1;
    cudaError_t enter(int dev) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) {
            prev = -1;
            return e;
        }
        return prev == dev ? cudaSuccess : cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

struct StaticRun {
    cudaStream_t s;
    int sms;
    bool table, dups;
    uint64_t level_cap;
    uint32_t* level[kMaxQ];
    uint32_t* defs;
    const uint32_t* nreq;
    uint32_t q;
    ExpandParams base;
    LaunchCtl* ctl;

    fm_status level_pass(uint32_t d, uint64_t n_parents, bool roots) {
        const int mode = (d == q - 1) ? (table ? kModeLastTable : kModeLastCount) : kModeMid;
        const int block = 256;
        const uint64_t n_chunks = (n_parents + 31) / 32;
        uint32_t* def_a = defs + (size_t)(2 * d) * kStaticDefCap;
        uint32_t* def_b = def_a + kStaticDefCap;
        uint32_t ndef_in = 0;
        uint64_t fresh = 0;
        const size_t smem = expand_smem_bytes(d, nreq[d], block / 32, 0);
        const int per_sm = expand_blocks_per_sm(mode, roots, dups, smem, block);
        // A launch defers at most 8 chunks per warp (the largest claim batch),
        // so a grid of at most kStaticDefCap / (8 * warps per block) blocks
        // keeps one launch's deferred chunks within a list whatever the SM
        // count; the carried-over entries are checked on the host below.
        const int def_bound = (int)(kStaticDefCap / (8u * (uint32_t)(block / 32)));
        const int full = std::max(1, std::min(std::min(sms * per_sm, sms * 2), def_bound));
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
            p.def_cap = kStaticDefCap;
            p.pout = (mode == kModeMid) ? level[d + 1] : nullptr;
            p.ocap = level_cap;
            const uint64_t want = (items + (block / 32) - 1) / (block / 32);
            int grid = (int)std::min<uint64_t>(want, (uint64_t)full);
            if (grid < 1) grid = 1;
            FM_CUDA(cudaMemsetAsync(ctl, 0, sizeof(LaunchCtl), s));
            FM_CUDA(launch_expand(p, mode, roots, dups, grid, full, block, smem, s));
            LaunchCtl c;
            FM_CUDA(cudaMemcpyAsync(&c, ctl, sizeof(LaunchCtl), cudaMemcpyDeviceToHost, s));
            FM_CUDA(cudaStreamSynchronize(s));
            if (c.error) {
                set_error("deferred-chunk list of the static scratch overflowed");
                return FM_ERR_DEVICE;
            }
            const uint64_t claimed = std::min<uint64_t>(c.claim, items);
            const uint64_t fresh_claimed = claimed > ndef_in ? claimed - ndef_in : 0;
            const uint64_t carry = ndef_in > claimed ? ndef_in - claimed : 0;
            fresh += fresh_claimed;
            uint64_t ndef_out = c.ndef;
            if (ndef_out + carry > kStaticDefCap) {
                set_error("deferred-chunk list of the static scratch overflowed");
                return FM_ERR_DEVICE;
            }
            if (carry) {
                FM_CUDA(cudaMemcpyAsync(def_b + ndef_out, def_a + claimed, carry * 4, cudaMemcpyDeviceToDevice, s));
                ndef_out += carry;
            }
            if (mode == kModeMid) {
                const uint64_t done_chunks = claimed - c.ndef;
                if (done_chunks == 0 && c.produced == 0 && ndef_out == items) {
                    set_error("a 32-parent chunk needs more rows than the static scratch holds");
                    return FM_ERR_POOL;
                }
                if (c.produced) {
                    fm_status st = level_pass(d + 1, c.produced, false);
                    if (st != FM_OK) return st;
                }
            }
            std::swap(def_a, def_b);
            ndef_in = (uint32_t)ndef_out;
        }
        return FM_OK;
    }
};

}  // namespace
}  // namespace fm

using namespace fm;

extern "C" fm_status fm_match_static(const fm_graph* graph, const fm_query* query, uint32_t* rows_out,
                                     uint64_t rows_cap, uint64_t* count_out, uint64_t* rows_written,
                                     void* stream) {
    if (!graph || !query || !count_out) return FM_ERR_ARG;
    *count_out = 0;
    if (rows_written) *rows_written = 0;
    const DeviceGraph& g = graph->g;
    const Plan& pl = query->p;
    // the caller's current device is restored on every return path
    DeviceGuard guard;
    FM_CUDA(guard.enter(g.device));
    unsigned char* scratch = nullptr;
    fm_status st = scratch_for_device(g.device, &scratch);
    if (st != FM_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t q = pl.q;
    const bool table = rows_out != nullptr;
    if (q < 2) {
        set_error("fm_match_static needs a query with at least two vertices");
        return FM_ERR_UNSUPPORTED;
    }
    if ((uint64_t)g.max_len * 32 >= (1ull << 32)) {
        set_error("a neighbour list is longer than 2^27");
        return FM_ERR_UNSUPPORTED;
    }

    // cost-based order (the reference's when the graph has duplicate e-lines)
    uint32_t order[kMaxQ], nreq[kMaxQ], climb[kMaxQ][kMaxQ], rlab[kMaxQ][kMaxQ];
    bool use_ref = g.has_dups != 0;
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
    uint32_t ref_depth[kMaxQ];
    for (uint32_t d = 0; d < q; d++) ref_depth[pl.order_local[d]] = d;

    StaticRun run;
    std::memset(&run.base, 0, sizeof(run.base));
    DevPlan& dp = run.base.plan;
    dp.q = q;
    uint32_t r = 0;
    for (uint32_t d = 0; d < q; d++) {
        dp.nreq[d] = nreq[d];
        dp.req_begin[d] = r;
        for (uint32_t i = 0; i < nreq[d]; i++, r++) {
            dp.req_anc[r] = (uint8_t)(d - climb[d][i]);
            dp.req_label[r] = (uint8_t)rlab[d][i];
            if (rlab[d][i] >= g.L) return FM_OK;   // a label absent from the graph: no embedding
        }
        dp.out_col[d] = (uint8_t)(q - 1 - ref_depth[order[d]]);   // the reference's column layout
        dp.col_depth[dp.out_col[d]] = (uint8_t)d;
    }

    // carve the static scratch: control blocks, deferred lists, heavy list, levels
    LaunchCtl* ctl = (LaunchCtl*)scratch;
    MatchTotals* tot = (MatchTotals*)(scratch + 512);
    uint32_t* defs = (uint32_t*)(scratch + kStaticCtlBytes);
    const uint64_t defs_bytes = 2ull * kMaxQ * kStaticDefCap * 4;
    HeavyEntry* heavy = (HeavyEntry*)(scratch + kStaticCtlBytes + defs_bytes);
    const uint64_t heavy_bytes = (uint64_t)kStaticHeavyCap * sizeof(HeavyEntry);
    const uint64_t level_base = kStaticCtlBytes + defs_bytes + heavy_bytes;
    const uint64_t level_bytes = kStaticScratchBytes - level_base;
    uint64_t sum_cols = 0;
    for (uint32_t d = 2; d < q; d++) sum_cols += d;
    uint64_t cap = sum_cols ? level_bytes / (4ull * sum_cols) : 0;
    if (sum_cols && cap < (uint64_t)g.max_len * 32 + 32) {
        set_error("query and graph need more partial-match room than the 64 MiB static scratch "
                  "of fm_match_static holds; use fm_match with a context");
        return FM_ERR_POOL;
    }
    int sms = 1;
    FM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g.device));
    run.s = s;
    run.sms = sms;
    run.table = table;
    run.dups = g.has_dups != 0;
    run.level_cap = cap;
    run.defs = defs;
    run.nreq = nreq;
    run.q = q;
    run.ctl = ctl;
    for (uint32_t d = 0; d < (uint32_t)kMaxQ; d++) run.level[d] = nullptr;
    uint64_t off = level_base;
    for (uint32_t d = 2; d < q; d++) {
        run.level[d] = (uint32_t*)(scratch + off);
        off += 4ull * d * cap;
    }
    ExpandParams& b = run.base;
    b.seg = g.seg;
    b.nbr = g.nbr;
    b.bm = g.bitmaps;
    b.bm_words = g.bm_words;
    b.V = g.V;
    b.root_begin = 0;
    b.table = rows_out;
    b.table_cap = table ? rows_cap : 0;
    b.table_vec4 = (table && q % 4 == 0 && ((uintptr_t)rows_out % 16) == 0) ? 1u : 0u;
    b.ctl = ctl;
    b.tot = tot;
    b.heavy = heavy;
    b.heavy_cap = kStaticHeavyCap;
    // the totals must start at zero: the scratch keeps the previous call's contents
    FM_CUDA(cudaMemsetAsync(tot, 0, sizeof(MatchTotals), s));
    st = run.level_pass(1, g.V, true);
    if (st != FM_OK) return st;
    MatchTotals t;
    FM_CUDA(cudaMemcpyAsync(&t, tot, sizeof(MatchTotals), cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaStreamSynchronize(s));
    *count_out = table ? t.table_pos : t.count;
    const uint64_t rows = table ? std::min<uint64_t>(*count_out, rows_cap) : 0;
    if (rows_written) *rows_written = rows;
    if (table && *count_out > rows_cap) {
        set_error("rows_out is smaller than the table; the count is exact");
        return FM_ERR_OUTPUT_OVERFLOW;
    }
    return FM_OK;
}
