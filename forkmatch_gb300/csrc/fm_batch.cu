// fm_batch.cu -- batched matching: many queries against one resident graph in
// shared level launches, captured once as a CUDA graph and replayed.
//
// The reference matches one query per program run (src/smsm.cu:1182-1349).
// Here a batch of queries advances level-synchronously: the level-d launch
// extends the partial matches of every query that is still open at depth d.
// Rows carry their query id in an extra column, every lane reads its own
// query's plan (requirements, table layout), and a survivor whose query ends
// at this depth goes straight to that query's count or table region, grouped
// per query with __match_any_sync (one atomic per query per warp round);
// survivors of longer queries are staged and flushed into the next level like
// in fm_match.cu.  So a batch needs max(q) - 1 level launches instead of
// sum(q - 1), and one host synchronisation.  Graphs with duplicate e-lines
// and single-vertex queries are matched one by one through fm_match.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <vector>

#include "fm_device.cuh"

namespace fm {

struct BatchPlan {                    // per query, in device memory
    uint32_t q;
    uint32_t nreq[kMaxQ];
    uint32_t req_begin[kMaxQ];
    uint8_t req_anc[kMaxReqTotal];
    uint8_t req_label[kMaxReqTotal];
    uint8_t col_depth[kMaxQ];         // depth whose vertex fills table column c
    uint64_t table_base;              // u32 offset of the query's table region
    uint64_t table_cap;               // rows
    uint64_t root_off;                // roots: heads[root_off .. root_off + n_roots)
    uint32_t n_roots;
    uint32_t count_only;              // no table for this query (count rule allowed)
    uint32_t pre_ok;                  // last depth has one back edge: when counting, depth q-2 counts
                                      // each survivor's extensions and depth q-1 is never reached
};

struct BatchParams {
    const BatchPlan* plans;
    uint32_t nq;
    const uint4* seg;
    const uint32_t* nbr;
    const uint32_t* bm;                       // list bitmaps (see DeviceGraph)
    uint32_t bm_words;
    uint32_t V;
    // parents: columns 0..d-1, query id in column d (null at depth 1: roots)
    const uint32_t* pin;
    uint64_t pstride;
    uint64_t n_parents;                       // roots: nq * chunks_per_query * 32
    const unsigned long long* n_parents_dev;  // set: read on the device (fresh chunks only)
    uint32_t chunks_per_query;                // roots: the longest root list, in 32-root chunks
    const uint32_t* heads;                    // per-label root lists of the graph
    uint32_t depth;
    uint32_t kmax;                            // segment records per parent reserved in shared memory
    // work items (deferred rings as in ExpandParams: def_in[(def_in_pos + i) %
    // def_cap], new deferrals at def_out_pos while fewer than def_room)
    const uint32_t* def_in;
    uint32_t ndef_in;
    uint64_t fresh_base;
    uint64_t n_items;
    uint32_t* def_out;
    uint32_t def_cap;
    uint64_t def_in_pos;
    uint64_t def_out_pos;
    uint32_t def_room;
    // outputs: next level (columns 0..d, query id in column d+1), per-query results
    uint32_t* pout;
    uint64_t ocap;
    uint32_t* table;
    unsigned long long* qpos;                 // per query: rows reserved (table) or count
    uint32_t table_mode;
    LaunchCtl* ctl;
    HeavyEntry* heavy;
    uint32_t heavy_cap;
    uint32_t max_warps;
    uint32_t piece_shift;                     // autotuned: heavy threshold and piece size scale
    uint32_t stage_words;                     // per-warp membership-list stage (0: lists stay in global memory)
    uint32_t self_loops;                      // the graph has an e-line v -> v (see ExpandParams)
};

namespace {

using dev::kFull;
using dev::ldg4;
using dev::seg_at;
using dev::seg_has;
using dev::slot_locate;

constexpr int kBWarps = 8;
constexpr uint32_t kBStage = 128;
constexpr uint32_t kBSlots = 2;            // candidate slots per lane per round
constexpr uint32_t kHeavyMaxPieces = 65536;

struct BTune {
    unsigned long long n_parents, n_items;
    uint32_t credit_block, heavy_thresh, heavy_piece;
    uint32_t claim_batch;    // chunks claimed per atomic (a level of 10^9 chunks must not serialise on one counter)
};

__device__ __forceinline__ BTune make_btune(const BatchParams& P) {
    BTune t;
    if (P.n_parents_dev) {
        t.n_parents = *(const volatile unsigned long long*)P.n_parents_dev;
        t.n_items = (t.n_parents + 31) / 32;
    } else {
        t.n_parents = P.n_parents;
        t.n_items = P.n_items;
    }
    const unsigned long long all_warps = P.max_warps ? P.max_warps : 1;
    const unsigned long long cb = P.ocap / (4 * all_warps);
    t.credit_block = (uint32_t)(cb < 1024 ? cb : 1024);
    const uint32_t base = t.n_items >= 4 * all_warps ? 2048u : (t.n_items >= all_warps ? 512u : 128u);
    t.heavy_piece = base << P.piece_shift;
    t.heavy_thresh = 2 * t.heavy_piece;
    // roots cost about the same per chunk: big batches; deeper chunks vary:
    // small batches keep the warps balanced
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x / 32);
    const unsigned long long b = (t.n_items / warps + 1) / (P.pin ? 16 : 2);
    t.claim_batch = (uint32_t)(b < 1 ? 1 : (b > 8 ? 8 : b));
    return t;
}

// Per-warp shared memory: rows, records, drivers, per-parent query data, stage.
struct BMem {
    uint32_t* rows_s;   // [d][32]
    uint4* segs_s;      // [kmax][32]
    uint32_t* excl_s;   // [32]
    uint32_t* drv_s;    // [32]
    uint32_t* k_s;      // [32] requirements of the parent's query at this depth
    uint32_t* qid_s;    // [32]
    uint32_t* pidx_s;   // [32] parent index in the level (root vertex at depth 1)
    uint32_t* fin_s;    // [32] 1: the parent's query ends at this depth; 2: it is pre-counted here
    uint32_t* stp;      // [kBStage] staged parent index
    uint32_t* stx;      // [kBStage] staged vertex
    uint32_t* stq;      // [kBStage] staged query id
    uint64_t* mbar;     // completion barrier of the list stage's bulk copies
    uint32_t* stage;    // [stage_words] membership lists copied in by TMA (optional)
};

__host__ __device__ constexpr uint32_t bper_warp_bytes(uint32_t d, uint32_t kmax, uint32_t stage_words = 0) {
    return 128 * d + 512 * kmax + 6 * 128 + 12 * kBStage + 4 * stage_words;
}

__device__ __forceinline__ BMem bmem(unsigned char* smem, uint32_t warp, uint32_t d, uint32_t kmax,
                                     uint32_t stage_words, uint64_t* mbar_s) {
    unsigned char* w = smem + warp * bper_warp_bytes(d, kmax, stage_words);
    BMem m;
    m.rows_s = (uint32_t*)w;
    m.segs_s = (uint4*)(w + 128 * d);
    uint32_t* s = (uint32_t*)(w + 128 * d + 512 * kmax);
    m.excl_s = s;
    m.drv_s = s + 32;
    m.k_s = s + 64;
    m.qid_s = s + 96;
    m.pidx_s = s + 128;
    m.fin_s = s + 160;
    m.stp = s + 192;
    m.stx = m.stp + kBStage;
    m.stq = m.stx + kBStage;
    m.mbar = mbar_s + warp;
    m.stage = (uint32_t*)(w + 128 * d + 512 * kmax + 6 * 128 + 12 * kBStage);
    return m;
}

constexpr uint32_t kBStageMaxList = 2048;
constexpr uint32_t kBStageSpinLimit = 1u << 22;

// Stage the membership lists of a loaded chunk into the warp's stage with
// TMA bulk copies (the same rule as the single-query kernel, with each lane's
// own number of back edges k and driver drv): non-driver lists of
// 4..kBStageMaxList entries without a bitmap whose copy pays for itself by
// the list-length ratio (dev::stage_worth), for parents with at least two
// candidates, lanes in order while the stage has room.  Returns false
// (warp-uniform) if the bounded wait ran out; error bit 2 is then raised.
__device__ __forceinline__ bool bstage_lists(const BatchParams& P, const BMem& m, uint32_t lane, uint32_t k,
                                             uint32_t drv, uint32_t n, bool valid, uint32_t sw, uint32_t& phase) {
    uint32_t want = 0;
    if (valid && k >= 2 && n >= 2) {
        for (uint32_t i = 0; i < k; i++) {
            if (i == drv) continue;
            const uint4 r = m.segs_s[i * 32 + lane];
            if (dev::stage_worth(r, n, kBStageMaxList)) want += (r.x + 3) & ~3u;
        }
    }
    uint32_t incl = want;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if ((int)lane >= o) incl += t;
    }
    const bool fits = want && incl <= sw;
    uint32_t bytes = fits ? want * 4 : 0;
#pragma unroll
    for (int o = 16; o; o >>= 1) bytes += __shfl_xor_sync(kFull, bytes, o);
    if (!bytes) return true;
    dev::fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) dev::mbar_arrive_expect_tx(m.mbar, bytes);
    __syncwarp();
    if (fits) {
        uint32_t off = incl - want;
        for (uint32_t i = 0; i < k; i++) {
            if (i == drv) continue;
            uint4 r = m.segs_s[i * 32 + lane];
            if (dev::stage_worth(r, n, kBStageMaxList)) {
                const uint32_t words = (r.x + 3) & ~3u;
                dev::bulk_copy_g2s(m.stage + off, P.nbr + (uint64_t)r.y * 4, words * 4, m.mbar);
                r.y = dev::kStagedMark | off;
                m.segs_s[i * 32 + lane] = r;
                off += words;
            }
        }
    }
    bool ok = false;
    for (uint32_t spin = 0; spin < kBStageSpinLimit && !ok; spin++) ok = dev::mbar_try_wait(m.mbar, phase);
    phase ^= 1u;
    ok = __all_sync(kFull, ok);
    if (!ok && lane == 0) atomicOr(&P.ctl->error, 2u);
    __syncwarp();
    return ok;
}

template <bool ROOTS>
__device__ __forceinline__ uint32_t bload_chunk(const BatchParams& P, const BMem& m, uint32_t chunk, uint32_t lane,
                                                uint32_t d, unsigned long long n_parents, bool& valid,
                                                uint32_t& k_out, unsigned long long& words, uint32_t sw,
                                                uint32_t& phase, bool& stage_ok, unsigned long long& rule_cnt,
                                                uint32_t& cont_total) {
    uint32_t qid, pidx;
    if (ROOTS) {
        qid = chunk / P.chunks_per_query;
        const uint32_t r = (chunk - qid * P.chunks_per_query) * 32 + lane;
        valid = qid < P.nq && r < P.plans[qid].n_roots;
        pidx = valid ? __ldg(P.heads + P.plans[qid].root_off + r) : 0u;   // the root vertex
        m.rows_s[lane] = pidx;
    } else {
        const uint64_t p = (uint64_t)chunk * 32 + lane;
        valid = p < n_parents;
        pidx = (uint32_t)p;
        qid = valid ? __ldg(P.pin + (uint64_t)d * P.pstride + p) : 0u;
        for (uint32_t c = 0; c < d; c++) m.rows_s[c * 32 + lane] = valid ? __ldg(P.pin + c * P.pstride + p) : 0u;
    }
    uint32_t n = 0, drv = 0, k = 0, fin = 0;
    words = 0;
    rule_cnt = 0;
    if (valid) {
        const BatchPlan& pl = P.plans[qid];
        k = pl.nreq[d];
        // bit 0: the query ends at this depth; bit 1: it is counted here (pre-count)
        fin = (pl.q == d + 1) ? 1u : 0u;
        if (pl.q == d + 2 && pl.pre_ok && (!P.table_mode || pl.count_only)) fin = 2u;
        const uint32_t rb = pl.req_begin[d];
        uint32_t best = 0xffffffffu;
        for (uint32_t i = 0; i < k; i++) {
            const uint32_t anc = pl.req_anc[rb + i];
            const uint32_t lab = pl.req_label[rb + i];
            const uint32_t v = m.rows_s[anc * 32 + lane];
            const uint4 sg = ldg4(P.seg + (uint64_t)lab * P.V + v);
            m.segs_s[i * 32 + lane] = sg;
            words += sg.x;
            if (sg.x < best) {
                best = sg.x;
                drv = i;
            }
        }
        n = best;
        if (k > 2) drv = dev::order_lists(m.segs_s, lane, k, drv);
        if (fin == 1u && k == 1 && (!P.table_mode || pl.count_only)) {
            // Count rule (the query's count only): every entry of the single
            // list extends the parent except the parent's own vertices, so the
            // extensions are counted, not enumerated.  The caller adds the
            // count once, when the main pass keeps the chunk (a chunk can be
            // loaded again after a deferral or for each heavy piece).
            const uint4 sg = m.segs_s[lane];
            rule_cnt = sg.x - dev::count_members(sg, m.rows_s, lane, d, 0u, false, P.nbr, P.bm, P.bm_words);
            n = 0;
        }
    }
    stage_ok = true;
    if (sw) stage_ok = bstage_lists(P, m, lane, k, drv, n, valid, sw, phase);
    k_out = k;
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if ((int)lane >= o) incl += t;
    }
    m.excl_s[lane] = incl - n;
    m.drv_s[lane] = drv;
    m.k_s[lane] = k;
    m.qid_s[lane] = qid;
    m.pidx_s[lane] = pidx;
    m.fin_s[lane] = fin;
    // candidate slots of the parents whose query goes on past this depth: the
    // only ones whose survivors can take rows of the next level
    cont_total = __reduce_add_sync(kFull, fin == 0u ? n : 0u);
    __syncwarp();
    return __shfl_sync(kFull, incl, 31);
}

// Staged survivors go to the next level; a parent's columns come from the
// warp's shared-memory copy of chunk `cur` when the parent belongs to it.
template <bool ROOTS>
__device__ __forceinline__ void bflush(const BatchParams& P, const BMem& m, uint32_t nst, uint32_t lane, uint32_t d,
                                       uint32_t cur) {
    unsigned long long pos0 = 0;
    if (lane == 0) pos0 = atomicAdd(&P.ctl->produced, (unsigned long long)nst);
    pos0 = __shfl_sync(kFull, pos0, 0);
    for (uint32_t c = 0; c < d; c++) {
        uint32_t* col = P.pout + c * P.ocap + pos0;
        for (uint32_t i = lane; i < nst; i += 32) {
            const uint32_t p = m.stp[i];
            col[i] = ROOTS ? p : ((p >> 5) == cur ? m.rows_s[c * 32 + (p & 31)] : __ldg(P.pin + c * P.pstride + p));
        }
    }
    uint32_t* colx = P.pout + d * P.ocap + pos0;
    uint32_t* colq = P.pout + (d + 1) * P.ocap + pos0;
    for (uint32_t i = lane; i < nst; i += 32) {
        colx[i] = m.stx[i];
        colq[i] = m.stq[i];
    }
}

// A survivor whose query ends at depth d+1: count it, or write its row into
// the query's table region.  Lanes of the same query share one atomic.
__device__ __forceinline__ void bfinal(const BatchParams& P, const BMem& m, bool okf, uint32_t j, uint32_t x,
                                       uint32_t lane, uint32_t d) {
    const unsigned fmask = __ballot_sync(kFull, okf);
    if (!fmask || !okf) return;
    const uint32_t qid = m.qid_s[j];
    const unsigned grp = __match_any_sync(fmask, qid);
    const int leader = __ffs(grp) - 1;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(&P.qpos[qid], (unsigned long long)__popc(grp));
    base = __shfl_sync(grp, base, leader);
    if (!P.table_mode) return;
    const BatchPlan& pl = P.plans[qid];
    const unsigned long long pos = base + __popc(grp & ((1u << lane) - 1u));
    if (pos >= pl.table_cap) return;
    uint32_t* o = P.table + pl.table_base + pos * pl.q;
    for (uint32_t c = 0; c < pl.q; c++) {
        const uint32_t dep = pl.col_depth[c];
        o[c] = dep < d ? m.rows_s[dep * 32 + j] : x;
    }
}

// A survivor counted by pre-count (its query's last depth has one back edge):
// its extensions are the entries of that list minus the row's vertices (the
// parent's and x) found in it.  Lanes of the same query share one atomic.
__device__ __forceinline__ void bprecount(const BatchParams& P, const BMem& m, bool pre, uint32_t j, uint32_t x,
                                          uint32_t lane, uint32_t d) {
    if (!__ballot_sync(kFull, pre)) return;
    uint32_t c = 0, qid = 0xffffffffu;
    if (pre) {
        qid = m.qid_s[j];
        const BatchPlan& pl = P.plans[qid];
        const uint32_t rb = pl.req_begin[d + 1];
        const uint32_t anc = pl.req_anc[rb];
        const uint4 sg = ldg4(P.seg + (uint64_t)pl.req_label[rb] * P.V + (anc == d ? x : m.rows_s[anc * 32 + j]));
        c = sg.x - dev::count_members(sg, m.rows_s, j, d, x, P.self_loops || anc != d, P.nbr, P.bm, P.bm_words);
    }
    const unsigned grp = __match_any_sync(kFull, qid);
    const unsigned lo = __reduce_add_sync(grp, c & 0xffffu);
    const unsigned hi = __reduce_add_sync(grp, c >> 16);
    if (pre && (int)lane == __ffs(grp) - 1 && (lo | hi))
        atomicAdd(&P.qpos[qid], ((unsigned long long)hi << 16) + lo);
}

// Evaluate slots [begin, end) of the loaded chunk, kBSlots per lane per round
// with every driver load of the round issued before any check (as in the
// single-query kernel); each slot's survivor is then counted or written
// (its query ends here), pre-counted, or staged for the next level.
template <bool ROOTS>
__device__ __forceinline__ void bprocess(const BatchParams& P, const BMem& m, uint32_t chunk, uint32_t begin,
                                         uint32_t end, uint32_t lane, uint32_t d, uint32_t& nst) {
    for (uint32_t base = begin; base < end; base += 32 * kBSlots) {
        uint32_t j[kBSlots], t[kBSlots], x[kBSlots];
        bool ok[kBSlots];
#pragma unroll
        for (uint32_t u = 0; u < kBSlots; u++) {
            const uint32_t s = base + 32 * u + lane;
            j[u] = t[u] = x[u] = 0;
            ok[u] = s < end;
            if (ok[u]) {
                slot_locate(s, m.excl_s, j[u], t[u]);
                x[u] = seg_at(m.segs_s[m.drv_s[j[u]] * 32 + j[u]], t[u], P.nbr);
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kBSlots; u++) {
            if (!ok[u]) continue;
            const uint32_t jj = j[u], dj = m.drv_s[jj], k = m.k_s[jj];
            for (uint32_t i = 0; i < k && ok[u]; i++) {
                if (i == dj) continue;
                ok[u] = dev::seg_has_st(m.segs_s[i * 32 + jj], x[u], 1, P.nbr, P.bm, P.bm_words, m.stage);
            }
            for (uint32_t c = 0; c < d && ok[u]; c++) ok[u] = m.rows_s[c * 32 + jj] != x[u];
        }
#pragma unroll
        for (uint32_t u = 0; u < kBSlots; u++) {
            const uint32_t fs = ok[u] ? m.fin_s[j[u]] : 0u;
            bfinal(P, m, fs == 1u, j[u], x[u], lane, d);
            bprecount(P, m, fs == 2u, j[u], x[u], lane, d);
            const bool stage = ok[u] && fs == 0u;
            const unsigned b = __ballot_sync(kFull, stage);
            if (stage) {
                const uint32_t q0 = nst + __popc(b & ((1u << lane) - 1u));
                m.stp[q0] = m.pidx_s[j[u]];
                m.stx[q0] = x[u];
                m.stq[q0] = m.qid_s[j[u]];
            }
            nst += __popc(b);
        }
        if (nst > kBStage - 32 * kBSlots) {
            __syncwarp();
            bflush<ROOTS>(P, m, nst, lane, d, chunk);
            nst = 0;
        }
        __syncwarp();
    }
}

__device__ __forceinline__ uint32_t bitem_chunk(const BatchParams& P, unsigned long long item) {
    return item < P.ndef_in ? P.def_in[(P.def_in_pos + item) % P.def_cap]
                            : (uint32_t)(P.fresh_base + (item - P.ndef_in));
}

__device__ __forceinline__ void bdefer(const BatchParams& P, uint32_t chunk) {
    const unsigned idx = atomicAdd(&P.ctl->ndef, 1u);
    const uint32_t room = P.def_room ? P.def_room : P.def_cap;
    if (idx < room) P.def_out[(P.def_out_pos + idx) % P.def_cap] = chunk;
    else atomicOr(&P.ctl->error, 1u);
}

template <bool ROOTS>
__device__ __forceinline__ void bexpand_main(const BatchParams& P, unsigned char* smem_raw, uint64_t* mbar_s,
                                             uint32_t& phase) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t d = P.depth;
    const uint32_t sw = P.kmax >= 2 ? P.stage_words : 0;   // only levels with membership tests stage lists
    const BMem m = bmem(smem_raw, threadIdx.x >> 5, d, P.kmax, sw, mbar_s);
    const BTune T = make_btune(P);
    unsigned long long n_lookups = 0, n_words = 0, n_parents = 0, credit = 0;
    uint32_t nst = 0;
    uint32_t last_chunk = 0xffffffffu;   // chunk whose rows are in m.rows_s
    bool done = false;
    while (!done) {
        unsigned long long first = 0;
        if (lane == 0) first = atomicAdd(&P.ctl->claim, (unsigned long long)T.claim_batch);
        first = __shfl_sync(kFull, first, 0);
        if (first >= T.n_items) break;
        const unsigned long long last = first + T.claim_batch < T.n_items ? first + T.claim_batch : T.n_items;
        for (unsigned long long item = first; item < last; item++) {
            const uint32_t chunk = bitem_chunk(P, item);
            int stop = 0;
            if (lane == 0) stop = *(volatile unsigned int*)&P.ctl->stop ? 1 : 0;
            stop = __shfl_sync(kFull, stop, 0);
            if (stop) {
                if (lane == 0)
                    for (unsigned long long it = item; it < last; it++) bdefer(P, bitem_chunk(P, it));
                done = true;
                break;
            }
            bool valid, stage_ok;
            uint32_t k;
            unsigned long long w, rule_cnt;
            uint32_t cont;
            const uint32_t total = bload_chunk<ROOTS>(P, m, chunk, lane, d, T.n_parents, valid, k, w, sw, phase,
                                                      stage_ok, rule_cnt, cont);
            last_chunk = chunk;
            if (!stage_ok) {
                done = true;
                break;
            }
            // only survivors of queries that go on use the next level's buffer:
            // the upper bound of their candidates is reserved (survivors that end
            // their query here, or are pre-counted, take no row)
            if (cont && P.pout) {
                int ok = 1;
                if (lane == 0 && cont > credit) {
                    const unsigned long long need =
                        max((unsigned long long)cont, (unsigned long long)T.credit_block);
                    const unsigned long long old = atomicAdd(&P.ctl->budget, need);
                    if (old + need > P.ocap) {
                        ok = 0;
                        atomicExch(&P.ctl->stop, 1u);
                        for (unsigned long long it = item; it < last; it++) bdefer(P, bitem_chunk(P, it));
                    } else {
                        credit += need;
                    }
                }
                if (lane == 0 && ok) credit -= cont;
                ok = __shfl_sync(kFull, ok, 0);
                if (!ok) {
                    done = true;
                    break;
                }
            }
            if (valid) {
                n_lookups += k;
                n_words += w;
                n_parents += 1;
            }
            {
                // count-rule counts: one atomic per query present in the chunk
                // (each lane's count is below 2^27, a warp's sum below 2^32)
                const uint32_t key = rule_cnt ? m.qid_s[lane] : 0xffffffffu;
                const unsigned grp = __match_any_sync(kFull, key);
                const unsigned sum = __reduce_add_sync(grp, (unsigned)rule_cnt);
                if (key != 0xffffffffu && (int)lane == __ffs(grp) - 1)
                    atomicAdd(&P.qpos[key], (unsigned long long)sum);
            }
            if (total > T.heavy_thresh) {
                int pub = 0;
                const uint32_t np = (total + T.heavy_piece - 1) / T.heavy_piece;
                if (lane == 0 && np <= kHeavyMaxPieces) {
                    const unsigned long long h = *(volatile unsigned long long*)&P.ctl->heavy;
                    if ((uint32_t)(h >> 32) + P.max_warps < P.heavy_cap && (uint32_t)h < (1u << 31)) {
                        const unsigned long long old = atomicAdd(&P.ctl->heavy, (1ull << 32) | np);
                        HeavyEntry e;
                        e.chunk = chunk;
                        e.total = total;
                        e.piece0 = (uint32_t)old;
                        e.pieces = np;
                        P.heavy[(uint32_t)(old >> 32)] = e;
                        pub = 1;
                    }
                }
                pub = __shfl_sync(kFull, pub, 0);
                if (pub) continue;
            }
            bprocess<ROOTS>(P, m, chunk, 0, total, lane, d, nst);
            // the stage refers to this chunk's query ids only through stq, and to
            // its parents through pidx: it can outlive the chunk
        }
    }
    if (nst) bflush<ROOTS>(P, m, nst, lane, d, last_chunk);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        n_lookups += __shfl_down_sync(kFull, n_lookups, o);
        n_words += __shfl_down_sync(kFull, n_words, o);
        n_parents += __shfl_down_sync(kFull, n_parents, o);
    }
    if (lane == 0 && n_parents) {
        atomicAdd(&P.ctl->parents, n_parents);
        atomicAdd(&P.ctl->lookups, n_lookups);
        atomicAdd(&P.ctl->list_words, n_words);
    }
}

template <bool ROOTS>
__device__ __forceinline__ void bexpand_heavy(const BatchParams& P, unsigned char* smem_raw, uint64_t* mbar_s,
                                              uint32_t& phase) {
    const unsigned long long h = *(volatile unsigned long long*)&P.ctl->heavy;
    const uint32_t nent = (uint32_t)(h >> 32);
    const uint32_t npieces = (uint32_t)h;
    if (nent == 0) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t d = P.depth;
    const uint32_t sw = P.kmax >= 2 ? P.stage_words : 0;
    const BMem m = bmem(smem_raw, threadIdx.x >> 5, d, P.kmax, sw, mbar_s);
    const BTune T = make_btune(P);
    uint32_t nst = 0;
    uint32_t last_chunk = 0xffffffffu;   // chunk whose rows are in m.rows_s
    for (;;) {
        unsigned long long gp = 0;
        if (lane == 0) gp = atomicAdd(&P.ctl->claim2, 1ull);
        gp = __shfl_sync(kFull, gp, 0);
        if (gp >= npieces) break;
        uint32_t lo = 0, hi = nent;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (P.heavy[mid].piece0 <= gp) lo = mid;
            else hi = mid;
        }
        const HeavyEntry e = P.heavy[lo];
        const uint32_t begin = ((uint32_t)gp - e.piece0) * T.heavy_piece;
        const uint32_t end = min(begin + T.heavy_piece, e.total);
        bool valid, stage_ok;
        uint32_t k;
        unsigned long long w, rule_cnt;   // counted by the main pass
        uint32_t cont;
        bload_chunk<ROOTS>(P, m, e.chunk, lane, d, T.n_parents, valid, k, w, sw, phase, stage_ok, rule_cnt, cont);
        last_chunk = e.chunk;
        if (!stage_ok) break;
        bprocess<ROOTS>(P, m, e.chunk, begin, end, lane, d, nst);
    }
    if (nst) bflush<ROOTS>(P, m, nst, lane, d, last_chunk);
}

template <bool ROOTS>
__global__ void __launch_bounds__(kBWarps * 32, 6) k_bexpand(const __grid_constant__ BatchParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t mbar_s[kBWarps];
    dev::stage_barriers_init(mbar_s);
    uint32_t phase = 0;
    bexpand_main<ROOTS>(P, smem_raw, mbar_s, phase);
}

template <bool ROOTS>
__global__ void __launch_bounds__(kBWarps * 32, 6) k_bexpand_heavy(const __grid_constant__ BatchParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t mbar_s[kBWarps];
    dev::stage_barriers_init(mbar_s);
    uint32_t phase = 0;
    bexpand_heavy<ROOTS>(P, smem_raw, mbar_s, phase);
}

// Persistent batch engine: one cooperative launch runs every level pass of
// the whole batch, scheduled on the device exactly like the single-query
// persistent kernel (fm_match.cu): per-depth work queues (deferred ring, then
// fresh chunks), depth-first drains, bounded grid barriers.
struct BatchPersistArgs {
    SchedState* sched;
    uint32_t* levels[kMaxQ];
    uint64_t caps[kMaxQ];             // rows of each level buffer
    uint32_t kmax[kMaxQ];
    uint32_t* rings;
    uint32_t ring_cap;
    uint32_t maxq;
    int hold_first_barrier;
};

__global__ void __launch_bounds__(kBWarps * 32, 5) k_bpersist(const __grid_constant__ BatchParams P0,
                                                              const __grid_constant__ BatchPersistArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) BatchParams P;
    __shared__ unsigned flag_s, cur_s;
    __shared__ uint64_t mbar_s[kBWarps];
    SchedState* S = A.sched;
    {
        const uint32_t* src = (const uint32_t*)&P0;
        uint32_t* dst = (uint32_t*)&P;
        for (uint32_t i = threadIdx.x; i < sizeof(BatchParams) / 4; i += blockDim.x) dst[i] = src[i];
    }
    dev::stage_barriers_init(mbar_s);
    uint32_t phase = 0;       // of this warp's stage barrier, carried across passes
    bool first = true;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned d = *(volatile unsigned*)&S->cur;
            if (*(volatile unsigned*)&S->error) d = 0;
            cur_s = d;
            if (d) {
                const volatile SchedLevel* L = &S->lv[d];
                const unsigned long long ring = L->tail - L->head;
                const unsigned long long n_chunks = (L->n_parents + 31) / 32;
                P.depth = d;
                P.kmax = A.kmax[d];
                P.pin = d == 1 ? nullptr : A.levels[d];
                P.pout = d + 1 < A.maxq ? A.levels[d + 1] : nullptr;
                P.pstride = d >= 2 ? A.caps[d] : 0;
                P.ocap = d + 1 < A.maxq ? A.caps[d + 1] : 0;
                P.n_parents = L->n_parents;
                P.ndef_in = (uint32_t)ring;
                P.fresh_base = L->fresh;
                P.n_items = ring + (n_chunks - L->fresh);
                P.def_in = A.rings + (uint64_t)d * A.ring_cap;
                P.def_out = A.rings + (uint64_t)d * A.ring_cap;
                P.def_cap = A.ring_cap;
                P.def_in_pos = L->head;
                P.def_out_pos = L->tail;
                P.def_room = A.ring_cap - (uint32_t)ring;
                P.ctl = P0.ctl + d;
            }
        }
        __syncthreads();
        const unsigned d = cur_s;
        if (d == 0) break;
        if (d == 1) bexpand_main<true>(P, smem_raw, mbar_s, phase);
        else bexpand_main<false>(P, smem_raw, mbar_s, phase);
        if (!dev::grid_barrier(S, first && A.hold_first_barrier && blockIdx.x == 0, &flag_s)) break;
        first = false;
        if (d == 1) bexpand_heavy<true>(P, smem_raw, mbar_s, phase);
        else bexpand_heavy<false>(P, smem_raw, mbar_s, phase);
        if (!dev::grid_barrier(S, false, &flag_s)) break;
        if (blockIdx.x == 0 && threadIdx.x == 0)
            dev::sched_advance(S, P0.ctl, d, d + 1 < A.maxq, P.n_items, P.ndef_in, P.def_room, false);
        if (!dev::grid_barrier(S, false, &flag_s)) break;
    }
}

int bpersist_blocks_per_sm(size_t smem) {
    allow_dynamic_smem((const void*)&k_bpersist);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, (const void*)&k_bpersist, kBWarps * 32, smem) !=
        cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    return n;
}

cudaError_t launch_bpersist(const BatchParams& p, const BatchPersistArgs& a, int grid, size_t smem,
                            cudaStream_t s) {
    BatchParams q = p;
    q.max_warps = (uint32_t)grid * kBWarps;
    q.n_parents_dev = nullptr;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kBWarps * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {(void*)&q, (void*)&a};
    return cudaLaunchKernelExC(&cfg, (const void*)&k_bpersist, args);
}

cudaError_t launch_batch_level(const BatchParams& p, bool roots, int grid, int heavy_grid, size_t smem,
                               cudaStream_t s) {
    void* f = roots ? (void*)&k_bexpand<true> : (void*)&k_bexpand<false>;
    void* fh = roots ? (void*)&k_bexpand_heavy<true> : (void*)&k_bexpand_heavy<false>;
    BatchParams q = p;
    q.max_warps = (uint32_t)heavy_grid * kBWarps;
    void* args[] = {(void*)&q};
    cudaError_t e = cudaLaunchKernel(f, dim3(grid), dim3(kBWarps * 32), args, smem, s);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernel(fh, dim3(heavy_grid), dim3(kBWarps * 32), args, smem, s);
}

int batch_blocks_per_sm(bool roots, size_t smem) {
    void* f = roots ? (void*)&k_bexpand<true> : (void*)&k_bexpand<false>;
    void* fh = roots ? (void*)&k_bexpand_heavy<true> : (void*)&k_bexpand_heavy<false>;
    allow_dynamic_smem(f);
    allow_dynamic_smem(fh);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, kBWarps * 32, smem) != cudaSuccess || n < 1) n = 1;
    return n;
}

}  // namespace
}  // namespace fm

// ------------------------------------------------------------------ host side

using namespace fm;

struct fm_batch {
    fm_context* ctx = nullptr;
    const fm_graph* graph = nullptr;
    uint32_t n = 0;
    int table = 0;
    std::vector<const fm_query*> queries;
    std::vector<uint32_t> batched;        // indices matched in the shared launches
    std::vector<uint32_t> single;         // indices matched one by one (q == 1, duplicate e-lines)
    std::vector<uint64_t> table_base, table_cap;
    BatchPlan* d_plans = nullptr;
    unsigned long long* d_qpos = nullptr;
    unsigned long long* h_qpos = nullptr;
    uint32_t maxq = 0;
    uint32_t kmax[kMaxQ] = {};
    uint64_t level_cap = 0;
    uint32_t* level[kMaxQ] = {};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};   // captured level sequence: count mode, table mode
    std::vector<BatchPlan> h_plans;                  // host copy (table regions are resized)
    bool regions_exact = false;                      // table regions sized from exact counts
    bool plans_dirty = false;                        // h_plans changed since the last upload
    bool replay = true;                              // capture the level sequence as a CUDA graph
    bool own_scratch = true;                         // d_plans, d_qpos, h_qpos allocated here

    void drop_graphs() {
        for (auto& e : exec) {
            if (e) cudaGraphExecDestroy(e);
            e = nullptr;
        }
    }
    uint32_t piece_shift = 0;
    uint32_t sm_fraction = 4;             // quarters of the full grid used by the main pass
    bool persistent = false;              // one cooperative launch per run (else level launches)
    bool graph_ok = true;                 // capture of the run succeeded (else launched directly)
    uint64_t cap_full = 0;                // largest level buffer (rows) SOLN_PREALLOC allows
    uint64_t cap_floor = 0;               // smallest level buffer one chunk per level needs
    uint32_t bank_shift = 0;              // tuned: level buffers of cap_full >> bank_shift rows
    char* soln = nullptr;

    uint64_t lcap[kMaxQ] = {};            // rows of the level buffer of depth d (d >= 2)
    uint64_t vol[kMaxQ] = {};             // rows that passed through level d in the last run
    bool weighted = false;                // level buffers sized from `vol` (else all equal)

    // Level buffers of `cap` rows each, packed from the start of the level region.
    void layout_levels(uint64_t cap) {
        weighted = false;
        level_cap = cap;
        uint64_t loff = 0;
        for (uint32_t d = 2; d < maxq; d++) {
            lcap[d] = cap;
            level[d] = (uint32_t*)(soln + loff);
            loff += 4ull * (d + 1) * cap;
        }
    }

    // Level buffers sized from the last run's per-depth volumes: a depth gets
    // room for all its rows when everything fits, else water-filling gives
    // every depth min(its volume, C) rows (never below one chunk's worth),
    // with C as large as SOLN_PREALLOC allows.  A batch whose queries stress
    // one depth (long paths) then drains it a few times instead of splitting
    // the memory evenly over every depth.  Returns false without volumes.
    bool layout_weighted() {
        uint64_t want[kMaxQ] = {};
        bool any = false;
        for (uint32_t d = 2; d < maxq; d++) {
            want[d] = std::max<uint64_t>(vol[d], cap_floor);
            any = any || vol[d] > 0;
        }
        if (!any) return false;
        const uint64_t budget = cap_full * ([&] {
            uint64_t c = 0;
            for (uint32_t d = 2; d < maxq; d++) c += 4ull * (d + 1);
            return c;
        }());
        auto bytes_at = [&](uint64_t C) {
            uint64_t t = 0;
            for (uint32_t d = 2; d < maxq; d++) t += 4ull * (d + 1) * std::max(cap_floor, std::min(want[d], C));
            return t;
        };
        uint64_t lo = cap_floor, hi = 0;
        for (uint32_t d = 2; d < maxq; d++) hi = std::max(hi, want[d]);
        if (bytes_at(lo) > budget) return false;
        while (lo < hi) {                      // largest C whose layout fits
            const uint64_t mid = lo + (hi - lo + 1) / 2;
            if (bytes_at(mid) <= budget) lo = mid;
            else hi = mid - 1;
        }
        weighted = true;
        uint64_t loff = 0;
        level_cap = 0;
        for (uint32_t d = 2; d < maxq; d++) {
            lcap[d] = std::min<uint64_t>(std::max(cap_floor, std::min(want[d], lo)), 0xffffffffull - 64);
            level_cap = std::max(level_cap, lcap[d]);
            level[d] = (uint32_t*)(soln + loff);
            loff += 4ull * (d + 1) * lcap[d];
        }
        return true;
    }
    std::vector<uint64_t> counts;
    std::vector<uint64_t> single_counts;
    uint64_t launches = 0;
    bool impossible_all = false;
    std::vector<uint8_t> impossible;      // a query label absent from the graph

    // Queries matched alone (tuned): a query whose work fills the GPU by
    // itself gains nothing from sharing launches and, in shared level
    // buffers, crowds out the others; it runs on the single-query engine
    // with the whole level memory, after the shared run, its table written
    // into its own region.  Indices are positions in `batched`.
    std::vector<uint8_t> solo;
    std::vector<uint32_t> roots_all;      // n_roots of every batched plan (solo plans get 0 in h_plans)
    uint32_t n_solo = 0;

    void set_solo(const std::vector<uint8_t>& s) {
        n_solo = 0;
        for (size_t i = 0; i < h_plans.size(); i++) {
            solo[i] = s[i];
            h_plans[i].n_roots = s[i] ? 0u : roots_all[i];
            n_solo += s[i] ? 1u : 0u;
        }
        plans_dirty = true;
        drop_graphs();                    // the captured launches bake in the longest root list
    }

    // The solo queries of one run: counted (count mode, or the counting run
    // that sizes table regions) or with their tables written into their
    // regions.  Their counts go to h_qpos like the shared run's.
    enum class SoloPick { All, CountOnly };
    fm_status run_solo(bool tables, SoloPick pick = SoloPick::All) {
        const ContextView cv = context_view(ctx);
        for (size_t i = 0; i < solo.size(); i++) {
            if (!solo[i]) continue;
            const BatchPlan& bp = h_plans[i];
            if (pick == SoloPick::CountOnly && !bp.count_only) continue;
            const bool tab = tables && !bp.count_only;
            fm_result r;
            const fm_status st = match_region(ctx, graph, queries[batched[i]], tab ? FM_MODE_TABLE : FM_MODE_COUNT,
                                              cv.output + bp.table_base, bp.table_cap, &r);
            if (st != FM_OK && st != FM_ERR_OUTPUT_OVERFLOW) return st;
            h_qpos[i] = r.count;
            launches += r.launches;
        }
        return FM_OK;
    }
};

namespace {

void build_plan(const Plan& pl, const DeviceGraph& g, BatchPlan& bp, bool& impossible) {
    std::memset(&bp, 0, sizeof(bp));
    const uint32_t q = pl.q;
    uint32_t order[kMaxQ], nreq[kMaxQ], climb[kMaxQ][kMaxQ], rlab[kMaxQ][kMaxQ];
    choose_order(pl, g, order);
    if (!order_requirements(pl, order, nreq, climb, rlab)) {
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
    bp.q = q;
    uint32_t r = 0;
    impossible = false;
    for (uint32_t d = 0; d < q; d++) {
        bp.nreq[d] = nreq[d];
        bp.req_begin[d] = r;
        for (uint32_t i = 0; i < nreq[d]; i++, r++) {
            bp.req_anc[r] = (uint8_t)(d - climb[d][i]);
            bp.req_label[r] = (uint8_t)rlab[d][i];
            if (rlab[d][i] >= g.L) impossible = true;
        }
        const uint32_t col = q - 1 - ref_depth[order[d]];
        bp.col_depth[col] = (uint8_t)d;
    }
    bp.pre_ok = (q >= 3 && nreq[q - 1] == 1 && pre_count_knob()) ? 1u : 0u;
    // roots: the vertices with an e-line of a depth-1 label (the shortest list)
    bool first = true;
    for (uint32_t i = 0; i < nreq[1] && !impossible; i++) {
        const uint32_t l = rlab[1][i];
        const uint64_t n = g.head_off[l + 1] - g.head_off[l];
        if (first || n < bp.n_roots) {
            bp.root_off = g.head_off[l];
            bp.n_roots = (uint32_t)n;
            first = false;
        }
    }
}

struct BatchRun {
    fm_batch* b;
    ContextView cv;
    const DeviceGraph* g;
    cudaStream_t s;
    BatchParams base;
    uint32_t nq;

    uint32_t* def_list(uint32_t d, int which) const {
        return cv.defs + (size_t)(2 * d + which) * cv.def_cap;
    }
    int gfull[kMaxQ] = {};
    size_t smem(uint32_t d) const {
        return (size_t)kBWarps * bper_warp_bytes(d, b->kmax[d], b->kmax[d] >= 2 ? base.stage_words : 0);
    }
    // occupancy queries and attribute changes happen here, before any capture
    void prepare() {
        for (uint32_t d = 1; d < b->maxq; d++) gfull[d] = cv.sms * batch_blocks_per_sm(d == 1, smem(d));
        pgrid = 0;
        if (b->persistent) {
            const int per_sm = bpersist_blocks_per_sm(psmem());
            if (per_sm > 0) pgrid = cv.sms * std::max(1, (per_sm * (int)b->sm_fraction + 3) / 4);
        }
    }
    int pgrid = 0;                        // persistent grid (0: level launches)
    size_t psmem() const {
        size_t m = 0;
        for (uint32_t d = 1; d < b->maxq; d++)
            m = std::max<size_t>(m, bper_warp_bytes(d, b->kmax[d], b->kmax[d] >= 2 ? base.stage_words : 0));
        return m * kBWarps;
    }

    // The persistent run as stream work (what the CUDA graph captures): clear
    // the per-query results and control blocks, write the initial schedule,
    // one cooperative launch, read back the schedule and the per-query results.
    fm_status enqueue_persist() {
        FM_CUDA(cudaMemsetAsync(b->d_qpos, 0, nq * sizeof(unsigned long long), s));
        FM_CUDA(cudaMemsetAsync(cv.ctl, 0, b->maxq * sizeof(LaunchCtl), s));
        FM_CUDA(launch_sched_init(cv.sched, b->maxq, (unsigned long long)nq * base.chunks_per_query * 32, 0,
                                  60000ull * 1000000ull, s));
        BatchParams p = base;
        p.ctl = cv.ctl;
        BatchPersistArgs a;
        std::memset(&a, 0, sizeof(a));
        a.sched = cv.sched;
        for (uint32_t d = 0; d < (uint32_t)kMaxQ; d++) {
            a.levels[d] = b->level[d];
            a.caps[d] = b->lcap[d];
            a.kmax[d] = b->kmax[d];
        }
        a.rings = cv.defs;
        a.ring_cap = 2 * cv.def_cap;
        a.maxq = b->maxq;
        FM_CUDA(launch_bpersist(p, a, pgrid, psmem(), s));
        FM_CUDA(cudaMemcpyAsync(cv.h_sched, cv.sched, sizeof(SchedState), cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaMemcpyAsync(b->h_qpos, b->d_qpos, nq * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        return FM_OK;
    }

    fm_status run_persist(bool use_graph) {
        bool ran = false;
        if (use_graph && b->graph_ok) {
            cudaGraphExec_t& exec = b->exec[base.table_mode ? 1 : 0];
            if (!exec) {
                cudaGraph_t graph = nullptr;
                FM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                fm_status st = enqueue_persist();
                cudaError_t e = cudaStreamEndCapture(s, &graph);
                if (st == FM_OK && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
                if (graph) cudaGraphDestroy(graph);
                if (st != FM_OK || e != cudaSuccess) {
                    // a cooperative launch this toolkit cannot capture: run it directly
                    cudaGetLastError();
                    exec = nullptr;
                    b->graph_ok = false;
                }
            }
            if (exec) {
                FM_CUDA(cudaGraphLaunch(exec, s));
                ran = true;
            }
        }
        if (!ran) FM_TRY(enqueue_persist());
        FM_CUDA(cudaStreamSynchronize(s));
        b->launches += 2;   // the schedule initialisation and the persistent kernel
        const SchedState& h = *cv.h_sched;
        for (uint32_t d = 0; d < (uint32_t)kMaxQ; d++) b->vol[d] = 0;
        for (uint32_t d = 1; d + 1 < b->maxq; d++) b->vol[d + 1] = h.lv[d].produced;
        if (h.error & kSchedErrWait) {
            set_error("a bounded wait of the persistent batch kernel ran out (a grid barrier or a list stage)");
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
        return FM_OK;
    }
    int full_grid(uint32_t d) const { return gfull[d]; }
    int main_grid(uint32_t d) const { return std::max(1, full_grid(d) * (int)b->sm_fraction / 4); }

    BatchParams level_params(uint32_t d) const {
        BatchParams p = base;
        p.depth = d;
        p.kmax = b->kmax[d];
        p.pin = d == 1 ? nullptr : b->level[d];
        p.pstride = d >= 2 ? b->lcap[d] : 0;
        p.pout = (d + 1 < b->maxq) ? b->level[d + 1] : nullptr;
        p.ocap = (d + 1 < b->maxq) ? b->lcap[d + 1] : 0;
        p.def_in = def_list(d, 0);
        p.def_out = def_list(d, 1);
        p.def_cap = cv.def_cap;
        p.ctl = cv.ctl + d;
        return p;
    }

    // Every level back to back; the stream work this enqueues is what the
    // CUDA graph captures.
    fm_status enqueue_all() {
        FM_CUDA(cudaMemsetAsync(b->d_qpos, 0, nq * sizeof(unsigned long long), s));
        for (uint32_t d = 1; d < b->maxq; d++) {
            BatchParams p = level_params(d);
            if (d == 1) {
                p.n_parents = (uint64_t)nq * base.chunks_per_query * 32;
                p.n_items = (uint64_t)nq * base.chunks_per_query;
            } else {
                p.n_parents_dev = &cv.ctl[d - 1].produced;
            }
            p.ndef_in = 0;
            p.fresh_base = 0;
            FM_CUDA(cudaMemsetAsync(cv.ctl + d, 0, sizeof(LaunchCtl), s));
            FM_CUDA(launch_batch_level(p, d == 1, main_grid(d), full_grid(d), smem(d), s));
        }
        FM_CUDA(cudaMemcpyAsync(cv.h_ctl, cv.ctl, b->maxq * sizeof(LaunchCtl), cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaMemcpyAsync(b->h_qpos, b->d_qpos, nq * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        return FM_OK;
    }

    // Host-driven depth-first drain of level d (same protocol as fm_match).
    fm_status drain(uint32_t d, uint64_t n_parents, uint32_t ndef_in, uint64_t fresh, uint32_t* def_a,
                    uint32_t* def_b) {
        const uint64_t n_chunks = d == 1 ? (uint64_t)nq * base.chunks_per_query : (n_parents + 31) / 32;
        while (true) {
            const uint64_t items = ndef_in + (n_chunks - fresh);
            if (items == 0) break;
            BatchParams p = level_params(d);
            p.n_parents = n_parents;
            p.n_items = items;
            p.def_in = def_a;
            p.ndef_in = ndef_in;
            p.fresh_base = fresh;
            p.def_out = def_b;
            FM_CUDA(cudaMemsetAsync(cv.ctl + d, 0, sizeof(LaunchCtl), s));
            const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((items + 7) / 8, (uint64_t)full_grid(d)));
            FM_CUDA(launch_batch_level(p, d == 1, grid, full_grid(d), smem(d), s));
            b->launches++;
            FM_CUDA(cudaMemcpyAsync(cv.h_ctl + d, cv.ctl + d, sizeof(LaunchCtl), cudaMemcpyDeviceToHost, s));
            FM_CUDA(cudaStreamSynchronize(s));
            const LaunchCtl c = cv.h_ctl[d];
            if (c.error) {
                set_error((c.error & 2u) ? "a list stage's bounded wait ran out" : "deferred-chunk list overflow");
                return FM_ERR_DEVICE;
            }
            const uint64_t claimed = std::min<uint64_t>(c.claim, items);
            const uint64_t fresh_claimed = claimed > ndef_in ? claimed - ndef_in : 0;
            const uint64_t carry = ndef_in > claimed ? ndef_in - claimed : 0;
            fresh += fresh_claimed;
            uint64_t ndef_out = c.ndef;
            if (ndef_out + carry > cv.def_cap) {
                set_error("deferred-chunk list overflow");
                return FM_ERR_DEVICE;
            }
            if (carry) {
                FM_CUDA(cudaMemcpyAsync(def_b + ndef_out, def_a + claimed, carry * 4, cudaMemcpyDeviceToDevice, s));
                ndef_out += carry;
            }
            if (d + 1 < b->maxq) {
                if (claimed - c.ndef == 0 && c.produced == 0 && ndef_out == items) {
                    set_error("one 32-parent chunk needs more rows than a level buffer holds; raise SOLN_PREALLOC");
                    return FM_ERR_POOL;
                }
                b->vol[d + 1] += c.produced;
                if (c.produced) FM_TRY(drain(d + 1, c.produced, 0, 0, def_list(d + 1, 0), def_list(d + 1, 1)));
            }
            std::swap(def_a, def_b);
            ndef_in = (uint32_t)ndef_out;
        }
        return FM_OK;
    }

    fm_status run(bool use_graph) {
        prepare();
        if (pgrid > 0) return run_persist(use_graph);
        if (use_graph) {
            cudaGraphExec_t& exec = b->exec[base.table_mode ? 1 : 0];
            if (!exec) {
                cudaGraph_t graph = nullptr;
                FM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                fm_status st = enqueue_all();
                cudaError_t e = cudaStreamEndCapture(s, &graph);
                if (st != FM_OK) {
                    if (graph) cudaGraphDestroy(graph);
                    return st;
                }
                if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
                e = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
            }
            FM_CUDA(cudaGraphLaunch(exec, s));
        } else {
            FM_TRY(enqueue_all());
        }
        FM_CUDA(cudaStreamSynchronize(s));
        b->launches += 2 * (b->maxq - 1);
        LaunchCtl snap[kMaxQ];
        std::memcpy(snap, cv.h_ctl, b->maxq * sizeof(LaunchCtl));
        uint64_t n_parents[kMaxQ] = {};
        for (uint32_t d = 0; d < (uint32_t)kMaxQ; d++) b->vol[d] = 0;
        for (uint32_t d = 1; d + 1 < b->maxq; d++) b->vol[d + 1] = snap[d].produced;
        for (uint32_t d = 1; d < b->maxq; d++) {
            if (snap[d].error) {
                set_error((snap[d].error & 2u) ? "a list stage's bounded wait ran out" : "deferred-chunk list overflow");
                return FM_ERR_DEVICE;
            }
            n_parents[d] = d == 1 ? (uint64_t)nq * base.chunks_per_query * 32 : snap[d - 1].produced;
        }
        bool resumed = false;
        for (uint32_t d = b->maxq - 1; d >= 1; d--) {
            if (d + 1 >= b->maxq) continue;   // the last level never defers
            const uint64_t items = d == 1 ? (uint64_t)nq * base.chunks_per_query : (n_parents[d] + 31) / 32;
            const uint64_t claimed = std::min<uint64_t>(snap[d].claim, items);
            if (snap[d].ndef == 0 && claimed == items) continue;
            resumed = true;
            FM_TRY(drain(d, n_parents[d], snap[d].ndef, claimed, def_list(d, 1), def_list(d, 0)));
        }
        if (resumed) {
            FM_CUDA(cudaMemcpyAsync(b->h_qpos, b->d_qpos, nq * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
            FM_CUDA(cudaStreamSynchronize(s));
        }
        return FM_OK;
    }
};

}  // namespace

namespace {

fm_status batch_create_impl(fm_context* ctx, const fm_graph* graph, const fm_query* const* queries, uint32_t n,
                            int32_t mode, const BatchScratch* scr, fm_batch** out) {
    if (!ctx || !graph || !out || (n && !queries)) return FM_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<fm_batch> b(new fm_batch());
    b->ctx = ctx;
    b->graph = graph;
    b->n = n;
    b->table = mode == FM_MODE_TABLE;
    b->queries.assign(queries, queries + n);
    b->counts.assign(n, 0);
    b->impossible.assign(n, 0);
    const DeviceGraph& g = graph->g;
    ContextView cv = context_view(ctx);
    if (cv.serving) {
        set_error("the context's slab belongs to a server (fm_server_create)");
        return FM_ERR_ARG;
    }
    if (g.device != cv.device) {
        set_error("graph and context live on different devices");
        return FM_ERR_ARG;
    }
    FM_CUDA(cudaSetDevice(cv.device));
    if ((uint64_t)g.max_len * 32 >= (1ull << 32)) {
        set_error("a neighbour list is longer than 2^27");
        return FM_ERR_UNSUPPORTED;
    }
    std::vector<BatchPlan> plans;
    uint64_t table_words = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (!queries[i]) return FM_ERR_ARG;
        const Plan& pl = queries[i]->p;
        if (pl.q < 2 || g.has_dups) {
            b->single.push_back(i);
            continue;
        }
        BatchPlan bp;
        bool imp = false;
        build_plan(pl, g, bp, imp);
        if (imp) {
            b->impossible[i] = 1;
            continue;
        }
        b->batched.push_back(i);
        plans.push_back(bp);
        table_words += pl.q;
    }
    // provisional table regions (the same number of rows for every batched
    // query); the first table run replaces them with exact ones
    const uint64_t rows_each = table_words ? cv.output_bytes / 4 / table_words : 0;
    uint64_t off = 0;
    for (auto& bp : plans) {
        bp.table_base = off;
        bp.table_cap = b->table ? rows_each : 0;
        off += rows_each * bp.q;
    }
    for (auto& bp : plans) {
        b->table_base.push_back(bp.table_base);
        b->table_cap.push_back(bp.table_cap);
        b->maxq = std::max(b->maxq, bp.q);
    }
    const uint32_t nq = (uint32_t)plans.size();
    if (nq) {
        for (uint32_t d = 1; d < b->maxq; d++) {
            uint32_t km = 1;
            for (auto& bp : plans)
                if (d < bp.q) km = std::max(km, bp.nreq[d]);
            b->kmax[d] = km;
        }
        uint64_t sum_cols = 0;   // level d+1 rows hold d+1 vertices and a query id
        for (uint32_t d = 2; d < b->maxq; d++) sum_cols += d + 1;
        uint64_t cap = sum_cols ? cv.soln_bytes / (4ull * sum_cols) : 0;
        cap = std::min<uint64_t>(cap, 0xffffffffull - 64);
        if (sum_cols && cap < (uint64_t)g.max_len * 32 + 32) {
            set_error("SOLN_PREALLOC cannot hold one 32-parent chunk per level for this graph");
            return FM_ERR_POOL;
        }
        b->soln = cv.soln;
        b->cap_full = cap;
        b->cap_floor = (uint64_t)g.max_len * 32 + 32;
        b->layout_levels(cap);
        b->h_plans = plans;
        b->solo.assign(nq, 0);
        for (auto& bp : plans) b->roots_all.push_back(bp.n_roots);
        if (scr) {
            // caller-owned scratch: no allocation (a server must not call
            // cudaMalloc/cudaFree while other slots run)
            if (scr->d_bytes < batch_scratch_bytes(nq, true) || scr->h_bytes < batch_scratch_bytes(nq, false)) {
                set_error("batch scratch too small");
                return FM_ERR_ARG;
            }
            b->own_scratch = false;
            b->d_plans = (BatchPlan*)scr->d;
            b->d_qpos = (unsigned long long*)((char*)scr->d + ((nq * sizeof(BatchPlan) + 255) & ~(size_t)255));
            b->h_qpos = (unsigned long long*)scr->h;
            FM_CUDA(cudaMemcpyAsync(b->d_plans, b->h_plans.data(), nq * sizeof(BatchPlan), cudaMemcpyHostToDevice,
                                    cv.stream));
        } else {
            FM_CUDA(cudaMalloc(&b->d_plans, nq * sizeof(BatchPlan)));
            FM_CUDA(cudaMemcpy(b->d_plans, plans.data(), nq * sizeof(BatchPlan), cudaMemcpyHostToDevice));
            FM_CUDA(cudaMalloc(&b->d_qpos, nq * sizeof(unsigned long long)));
            FM_CUDA(cudaHostAlloc(&b->h_qpos, nq * sizeof(unsigned long long), cudaHostAllocDefault));
        }
    }
    *out = b.release();
    return FM_OK;
}

}  // namespace

size_t fm::batch_scratch_bytes(uint32_t n, bool device) {
    if (!device) return (size_t)n * sizeof(unsigned long long);
    return ((n * sizeof(BatchPlan) + 255) & ~(size_t)255) + (size_t)n * sizeof(unsigned long long);
}

fm_status fm::batch_create_scratch(fm_context* ctx, const fm_graph* graph, const fm_query* const* queries, uint32_t n,
                                   int32_t mode, const BatchScratch& scratch, fm_batch** out) {
    return batch_create_impl(ctx, graph, queries, n, mode, &scratch, out);
}

extern "C" {

fm_status fm_batch_create(fm_context* ctx, const fm_graph* graph, const fm_query* const* queries, uint32_t n,
                          int32_t mode, fm_batch** out) {
    return batch_create_impl(ctx, graph, queries, n, mode, nullptr, out);
}

void fm_batch_free(fm_batch* b) {
    if (!b) return;
    b->drop_graphs();
    if (b->own_scratch) {
        if (b->d_plans) cudaFree(b->d_plans);
        if (b->d_qpos) cudaFree(b->d_qpos);
        if (b->h_qpos) cudaFreeHost(b->h_qpos);
    }
    delete b;
}

fm_status fm_batch_run(fm_batch* b, uint64_t* counts, fm_batch_stats* stats) {
    if (!b) return FM_ERR_ARG;
    ContextView cv = context_view(b->ctx);
    FM_CUDA(cudaSetDevice(cv.device));
    auto t0 = std::chrono::steady_clock::now();
    const uint64_t launches0 = b->launches;
    const DeviceGraph& g = b->graph->g;
    const uint32_t nq = (uint32_t)b->batched.size();
    int truncated = 0;
    if (nq) {
        BatchRun run;
        run.b = b;
        run.cv = cv;
        run.g = &g;
        run.s = cv.stream;
        run.nq = nq;
        std::memset(&run.base, 0, sizeof(run.base));
        run.base.plans = b->d_plans;
        run.base.nq = nq;
        run.base.seg = g.seg;
        run.base.nbr = g.nbr;
        run.base.bm = g.bitmaps;
        run.base.bm_words = g.bm_words;
        run.base.V = g.V;
        uint32_t longest = 1;
        for (const BatchPlan& bp : b->h_plans) longest = std::max(longest, bp.n_roots);
        run.base.chunks_per_query = (longest + 31) / 32;
        run.base.heads = g.heads;
        run.base.table = cv.output;
        run.base.qpos = b->d_qpos;
        run.base.heavy = cv.heavy;
        run.base.heavy_cap = cv.heavy_cap;
        run.base.piece_shift = b->piece_shift;
        run.base.stage_words = stage_words_knob();
        run.base.self_loops = g.has_self_loops ? 1u : 0u;
        if ((uint64_t)nq * run.base.chunks_per_query >= (1ull << 32)) {
            set_error("too many (query, root chunk) pairs in one batch; split the batch");
            return FM_ERR_UNSUPPORTED;
        }
        if (b->plans_dirty) {
            FM_CUDA(cudaMemcpyAsync(b->d_plans, b->h_plans.data(), nq * sizeof(BatchPlan), cudaMemcpyHostToDevice,
                                    cv.stream));
            b->plans_dirty = false;
        }
        // done[i]: query i's result is already final in this (first table) run
        std::vector<uint8_t> done;
        std::vector<uint64_t> first_counts;
        if (b->table && !b->regions_exact) {
            // First table run: count the queries of the shared launches and
            // the count-only queries matched alone, give each shared table
            // query a table region of exactly its size (in order, while
            // OUTPUT_PREALLOC lasts), then match the table queries matched
            // alone in table mode once, each straight into the free space
            // after the last region (its region is what it wrote).
            run.base.table_mode = 0;
            FM_TRY(run.run(b->replay));
            FM_TRY(b->run_solo(false, fm_batch::SoloPick::CountOnly));
            const uint64_t words = cv.output_bytes / 4;
            uint64_t off = 0;
            for (uint32_t i = 0; i < nq; i++) {
                BatchPlan& bp = b->h_plans[i];
                if (b->solo[i] && !bp.count_only) continue;
                const uint64_t need = bp.count_only ? 0 : b->h_qpos[i] * bp.q;
                bp.table_base = off;
                bp.table_cap = (!bp.count_only && off + need <= words) ? b->h_qpos[i] : 0;
                off += bp.table_cap * bp.q;
            }
            for (uint32_t i = 0; i < nq; i++) {
                BatchPlan& bp = b->h_plans[i];
                if (!b->solo[i] || bp.count_only) continue;
                bp.table_base = off;
                bp.table_cap = (words - off) / bp.q;
                fm_result r;
                const fm_status st = match_region(b->ctx, b->graph, b->queries[b->batched[i]], FM_MODE_TABLE,
                                                  cv.output + off, bp.table_cap, &r);
                if (st != FM_OK && st != FM_ERR_OUTPUT_OVERFLOW) return st;
                b->launches += r.launches;
                b->h_qpos[i] = r.count;
                bp.table_cap = std::min<uint64_t>(bp.table_cap, r.count);
                off += bp.table_cap * bp.q;
            }
            for (uint32_t i = 0; i < nq; i++) {
                b->table_base[i] = b->h_plans[i].table_base;
                b->table_cap[i] = b->h_plans[i].table_cap;
            }
            // Count-only queries are exact after the counting run and the
            // table queries matched alone are written: the table pass below
            // skips both (shared ones by withholding their roots; it is
            // launched directly, not captured, since its plans differ from
            // later runs').
            first_counts.assign(b->h_qpos, b->h_qpos + nq);
            done.assign(nq, 0);
            for (uint32_t i = 0; i < nq; i++) {
                done[i] = (b->h_plans[i].count_only || b->solo[i]) ? 1 : 0;
                if (b->h_plans[i].count_only) b->h_plans[i].n_roots = 0;
            }
            FM_CUDA(cudaMemcpyAsync(b->d_plans, b->h_plans.data(), nq * sizeof(BatchPlan), cudaMemcpyHostToDevice,
                                    cv.stream));
            b->regions_exact = true;
        }
        run.base.table_mode = b->table ? 1u : 0u;
        FM_TRY(run.run(b->replay && done.empty()));
        if (done.empty()) {
            FM_TRY(b->run_solo(b->table != 0, fm_batch::SoloPick::All));
        } else {
            for (uint32_t i = 0; i < nq; i++) {
                if (!done[i]) continue;
                b->h_qpos[i] = first_counts[i];
                b->h_plans[i].n_roots = b->solo[i] ? 0u : b->roots_all[i];
            }
            b->plans_dirty = true;
        }
        for (uint32_t i = 0; i < nq; i++) {
            const uint32_t qi = b->batched[i];
            b->counts[qi] = b->h_qpos[i];
            if (b->table && !b->h_plans[i].count_only && b->h_qpos[i] > b->table_cap[i]) truncated = 1;
        }
    }
    for (uint32_t qi = 0; qi < b->n; qi++)
        if (b->impossible[qi]) b->counts[qi] = 0;
    // queries matched one by one (q == 1, or a graph with duplicate e-lines)
    b->single_counts.clear();
    for (uint32_t qi : b->single) {
        fm_match_opts o;
        fm_match_opts_default(&o);
        o.mode = FM_MODE_COUNT;
        fm_result r;
        fm_status st = fm_match(b->ctx, b->graph, b->queries[qi], &o, &r);
        if (st != FM_OK) return st;
        b->counts[qi] = r.count;
        b->launches += r.launches;
    }
    if (counts)
        for (uint32_t i = 0; i < b->n; i++) counts[i] = b->counts[i];
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->launches = b->launches - launches0;
        stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->batched_queries = nq;
        stats->single_queries = (uint32_t)b->single.size();
        stats->piece_shift = b->piece_shift;
        stats->grid_quarters = b->sm_fraction;
        stats->level_rows = b->level_cap;
        stats->persistent = b->persistent ? 1 : 0;
        stats->graph = (b->replay && b->graph_ok) ? 1 : 0;
        stats->weighted_levels = b->weighted ? 1 : 0;
        stats->solo_queries = (int32_t)b->n_solo;
        for (uint32_t i = 0; i < b->n; i++) stats->embeddings += b->counts[i];
    }
    if (truncated) {
        set_error("a query's table region overflowed; counts are exact");
        return FM_ERR_OUTPUT_OVERFLOW;
    }
    return FM_OK;
}

fm_status fm_batch_rows(const fm_batch* b, uint32_t i, const uint32_t** rows_device, uint64_t* rows) {
    if (!b || i >= b->n || !rows_device || !rows) return FM_ERR_ARG;
    *rows_device = nullptr;
    *rows = 0;
    if (!b->table) return FM_OK;
    for (size_t k = 0; k < b->batched.size(); k++) {
        if (b->batched[k] != i) continue;
        ContextView cv = context_view(b->ctx);
        *rows_device = cv.output + b->table_base[k];
        *rows = std::min<uint64_t>(b->counts[i], b->table_cap[k]);
        return FM_OK;
    }
    set_error("this query was matched on its own (no batch table region)");
    return FM_ERR_ARG;
}

fm_status fm_batch_copy_rows(const fm_batch* b, uint32_t i, uint32_t* host, uint64_t cap, uint64_t* copied) {
    if (!copied || (cap && !host)) return FM_ERR_ARG;
    *copied = 0;
    const uint32_t* rows_device = nullptr;
    uint64_t rows = 0;
    FM_TRY(fm_batch_rows(b, i, &rows_device, &rows));
    const uint64_t n = std::min(rows, cap);
    if (n) {
        ContextView cv = context_view(b->ctx);
        FM_CUDA(cudaMemcpyAsync(host, rows_device, n * b->queries[i]->p.q * 4, cudaMemcpyDeviceToHost, cv.stream));
        FM_CUDA(cudaStreamSynchronize(cv.stream));
    }
    *copied = n;
    return FM_OK;
}

}  // extern "C"

void fm::batch_set_replay(fm_batch* b, bool replay) {
    // a server's batches run once, beside other slots' work: no capture, and
    // level launches (a cooperative launch needs the whole GPU resident)
    if (b) {
        b->replay = replay;
        if (!replay) b->persistent = false;
    }
}

extern "C" {

fm_status fm_batch_copy_tables(const fm_batch* b, uint32_t* host, uint64_t cap_words, uint64_t* offsets,
                               uint64_t* words) {
    if (!b || !words || (cap_words && !host)) return FM_ERR_ARG;
    *words = 0;
    if (offsets)
        for (uint32_t i = 0; i < b->n; i++) offsets[i] = UINT64_MAX;
    if (!b->table || b->batched.empty()) return FM_OK;
    // regions are disjoint; the packed span ends after the last region that
    // holds rows
    uint64_t end = 0;
    for (size_t k = 0; k < b->batched.size(); k++) {
        const uint32_t qi = b->batched[k];
        const uint64_t rows = std::min<uint64_t>(b->counts[qi], b->table_cap[k]);
        if (offsets) offsets[qi] = b->table_base[k];
        end = std::max<uint64_t>(end, b->table_base[k] + rows * b->queries[qi]->p.q);
    }
    if (end > cap_words) {
        set_error("host buffer smaller than the batch tables");
        return FM_ERR_OUTPUT_OVERFLOW;
    }
    if (end) {
        ContextView cv = context_view(b->ctx);
        FM_CUDA(cudaSetDevice(cv.device));
        FM_CUDA(cudaMemcpyAsync(host, cv.output, end * 4, cudaMemcpyDeviceToHost, cv.stream));
        FM_CUDA(cudaStreamSynchronize(cv.stream));
    }
    *words = end;
    return FM_OK;
}

fm_status fm_batch_set_query_mode(fm_batch* b, uint32_t i, int32_t mode) {
    if (!b || i >= b->n || (mode != FM_MODE_TABLE && mode != FM_MODE_COUNT)) return FM_ERR_ARG;
    for (size_t k = 0; k < b->batched.size(); k++) {
        if (b->batched[k] != i) continue;
        const uint32_t co = mode == FM_MODE_COUNT ? 1u : 0u;
        if (b->h_plans[k].count_only != co) {
            b->h_plans[k].count_only = co;
            b->plans_dirty = true;
            b->regions_exact = false;
            b->drop_graphs();
        }
    }
    return FM_OK;   // queries matched on their own are counted only anyway
}

fm_status fm_batch_set_engine(fm_batch* b, int32_t engine) {
    if (!b || (engine != FM_ENGINE_PERSISTENT && engine != FM_ENGINE_LEVELS)) return FM_ERR_ARG;
    if (!b->replay && engine == FM_ENGINE_PERSISTENT) {
        set_error("a server's batches use level launches");
        return FM_ERR_ARG;
    }
    b->persistent = engine == FM_ENGINE_PERSISTENT;
    b->drop_graphs();
    return FM_OK;
}

fm_status fm_batch_set_solo(fm_batch* b, uint32_t i, int32_t solo) {
    if (!b || i >= b->n) return FM_ERR_ARG;
    for (size_t k = 0; k < b->batched.size(); k++) {
        if (b->batched[k] != i || (b->solo[k] != 0) == (solo != 0)) continue;
        std::vector<uint8_t> s = b->solo;
        s[k] = solo ? 1 : 0;
        b->set_solo(s);
    }
    return FM_OK;
}

fm_status fm_batch_get_solo(const fm_batch* b, uint32_t i, int32_t* solo) {
    if (!b || i >= b->n || !solo) return FM_ERR_ARG;
    *solo = 0;
    for (size_t k = 0; k < b->batched.size(); k++)
        if (b->batched[k] == i) *solo = b->solo[k];
    return FM_OK;
}

fm_status fm_batch_tune(fm_batch* b, fm_batch_stats* best) {
    if (!b) return FM_ERR_ARG;
    // First the queries matched alone: every batched query is timed alone on
    // the single-query engine, and a query runs alone when that time is at
    // least a threshold (8 ms or 2 ms: its work fills the GPU by itself);
    // each threshold's batch is timed on a replay after its capturing run,
    // and the fastest set (possibly none) is kept.
    // Then, with that set, the engine, the split granularity (heavy piece
    // size: the intersection tile a warp walks), the grid (warps in flight
    // per SM) and the level-buffer size (rows per buffer, the bank size:
    // small buffers keep the rows of a depth-first drain in L2, large or
    // volume-weighted ones need fewer passes): both engines at the full grid
    // and full level buffers, then for the level engine the split
    // granularity, a half grid, smaller and volume-weighted level buffers.
    // Each candidate runs the whole batch once (capturing its graph, which
    // that run then launches) and is timed on that run; the fastest is kept.
    if (b->replay && !b->batched.empty()) {      // a server's batches share their launches
        const size_t nb = b->batched.size();
        b->set_solo(std::vector<uint8_t>(nb, 0));
        b->layout_levels(b->cap_full >> b->bank_shift);
        fm_batch_stats st0;
        fm_status s0 = fm_batch_run(b, nullptr, &st0);    // sizes the table regions, captures
        if (s0 != FM_OK && s0 != FM_ERR_OUTPUT_OVERFLOW) return s0;
        s0 = fm_batch_run(b, nullptr, &st0);
        if (s0 != FM_OK && s0 != FM_ERR_OUTPUT_OVERFLOW) return s0;
        const ContextView cv = context_view(b->ctx);
        std::vector<double> alone(nb, 0.0);
        for (size_t i = 0; i < nb; i++) {
            const BatchPlan& bp = b->h_plans[i];
            const bool tab = b->table && !bp.count_only;
            fm_result r;
            const fm_status st = match_region(b->ctx, b->graph, b->queries[b->batched[i]],
                                              tab ? FM_MODE_TABLE : FM_MODE_COUNT, cv.output + bp.table_base,
                                              bp.table_cap, &r);
            if (st != FM_OK && st != FM_ERR_OUTPUT_OVERFLOW) return st;
            alone[i] = r.device_ms;
        }
        double solo_best = st0.wall_ms;
        std::vector<uint8_t> solo_pick(nb, 0);
        for (const double tau : {8.0, 2.0}) {
            std::vector<uint8_t> sv(nb, 0);
            bool any = false;
            for (size_t i = 0; i < nb; i++) any |= (sv[i] = alone[i] >= tau ? 1 : 0) != 0;
            if (!any || sv == solo_pick) continue;
            b->set_solo(sv);
            fm_batch_stats st;
            fm_status s1 = fm_batch_run(b, nullptr, &st);     // captures the shared part
            if (s1 != FM_OK && s1 != FM_ERR_OUTPUT_OVERFLOW) return s1;
            s1 = fm_batch_run(b, nullptr, &st);
            if (s1 != FM_OK && s1 != FM_ERR_OUTPUT_OVERFLOW) return s1;
            if (st.wall_ms < solo_best) {
                solo_best = st.wall_ms;
                solo_pick = sv;
            }
        }
        b->set_solo(solo_pick);
    }
    struct Cand {
        bool persistent;
        uint32_t shift, quarters, bank;
    };
    // bank kWeighted: level buffers sized from the previous run's per-depth volumes
    constexpr uint32_t kWeighted = 99;
    std::vector<Cand> cands = {{false, 0, 4, 0}, {true, 0, 4, 0}, {false, 1, 4, 0}, {false, 0, 2, 0},
                               {false, 0, 4, 4}, {false, 0, 4, kWeighted}};
    uint64_t vol0[kMaxQ];
    std::memcpy(vol0, b->vol, sizeof(vol0));
    bool have_vol = false;
    for (uint32_t d = 2; d < b->maxq; d++) have_vol = have_vol || vol0[d] > 0;
    if (!b->replay) cands.erase(cands.begin() + 1);   // a server's batches use level launches
    double best_ms = -1;
    Cand best_c = {b->persistent, b->piece_shift, b->sm_fraction, b->bank_shift};
    for (const Cand& c : cands) {
        if (c.bank == kWeighted) {
            if (!have_vol) continue;
        } else if (c.bank && (b->cap_full >> c.bank) < b->cap_floor) {
            continue;
        }
        b->persistent = c.persistent;
        b->piece_shift = c.shift;
        b->sm_fraction = c.quarters;
        b->bank_shift = c.bank;
        if (c.bank == kWeighted) {
            std::memcpy(b->vol, vol0, sizeof(vol0));
            if (!b->layout_weighted()) continue;
        } else {
            b->layout_levels(b->cap_full >> c.bank);
        }
        b->drop_graphs();
        fm_batch_stats st;
        fm_status s = fm_batch_run(b, nullptr, &st);
        if (s != FM_OK && s != FM_ERR_OUTPUT_OVERFLOW) return s;
        if (best_ms < 0 || st.wall_ms < best_ms) {
            best_ms = st.wall_ms;
            best_c = c;
        }
    }
    b->persistent = best_c.persistent;
    const uint32_t bs = best_c.shift, bq = best_c.quarters, bb = best_c.bank;
    b->piece_shift = bs;
    b->sm_fraction = bq;
    b->bank_shift = bb;
    if (bb == kWeighted) {
        std::memcpy(b->vol, vol0, sizeof(vol0));
        if (!b->layout_weighted()) b->layout_levels(b->cap_full);
    } else {
        b->layout_levels(b->cap_full >> bb);
    }
    b->drop_graphs();
    if (best) {
        std::memset(best, 0, sizeof(*best));
        best->wall_ms = best_ms;
        best->piece_shift = bs;
        best->grid_quarters = bq;
        best->level_rows = b->level_cap;
        best->persistent = b->persistent ? 1 : 0;
        best->graph = b->graph_ok ? 1 : 0;
        best->weighted_levels = b->weighted ? 1 : 0;
        best->solo_queries = (int32_t)b->n_solo;
    }
    return FM_OK;
}

}  // extern "C"
