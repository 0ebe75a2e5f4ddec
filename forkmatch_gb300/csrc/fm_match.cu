// fm_match.cu -- level-expansion kernels of the matcher.
//
// Replaces the reference's per-thread k-way merge (src/smsm.cu:299-345 isoGen,
// src/smsm.cu:57-140 isoCompare), injectivity walk (src/smsm.cu:188-227 isInj),
// ballot append (src/smsm.cu:146-182 attemptInsert) and table write
// (src/smsm.cu:706-779 isoWrite).
//
// One level launch extends every partial match by one query vertex.  Partial
// matches are full rows (column c = data vertex matched at depth c) stored
// column-major (SoA), so every load and store of a column is coalesced; there
// is no parent-pointer forest to climb.  Warps claim chunks of 32 parents
// (several chunks per atomic):
//   1. each lane loads its parent row and the k (label, ancestor) segment
//      records -- k independent 16-byte loads, issued back to back;
//   2. the shortest list is the driver; a warp prefix sum over driver lengths
//      turns the 32 parents' candidate lists into one range of slots;
//   3. lanes take 64 consecutive slots per round, two per lane with both driver
//      loads in flight (load-balanced across parents, so a hub parent keeps all
//      32 lanes busy), reject values already in the row, test membership in
//      the other k-1 lists (inline compare or binary search), and stage
//      survivors as (parent index, value) in shared memory;
//   4. the stage outlives the chunk: it is flushed with one atomic per 448+
//      survivors and fully coalesced stores, column by column into the next
//      level or as contiguous row-major rows into the table.
// A chunk whose candidate range is long (a hub) is not walked by one warp: it
// is published to a heavy list and cut into pieces that every warp of a second
// launch shares.  Lists of length <= 3 are inline in the segment record, so
// the common case needs no second memory access.  With duplicate e-lines the
// value at rank r of its run in the driver list survives only if every other
// list holds at least r + 1 copies (min-multiplicity semantics of the
// reference's merge).
//
// Bounded memory: before expanding a chunk a warp holds output budget for its
// candidate upper bound (reserved from the level in blocks); when a
// reservation does not fit, the warp defers its remaining chunks, raises
// `stop`, and exits; the host drains the output level (depth first) and
// relaunches this level on the deferred chunks plus the unclaimed remainder.
// Nothing spins and nothing traps.
#include <algorithm>
#include <mutex>
#include <set>
#include <utility>

#include "fm_device.cuh"

namespace fm {
namespace {

using dev::kFull;
using dev::ldg4;
using dev::lower_bound_g;
using dev::seg_at;
using dev::seg_has;
using dev::slot_locate;

constexpr int kWarps = 8;
constexpr uint32_t kStage = 256;           // staged survivors per warp
constexpr uint32_t kSlots = 2;             // candidate slots per lane per round
constexpr uint32_t kHeavyMaxPieces = 65536;

// Rank of position t within its run of equal values.
__device__ __forceinline__ uint32_t seg_rank(const uint4& s, uint32_t t, uint32_t x, const uint32_t* __restrict__ nbr) {
    if (s.x <= 3) return (t >= 1 && s.y == x) + (t >= 2 && s.z == x);
    const uint32_t* a = nbr + (uint64_t)s.y * 4;
    return t - lower_bound_g(a, t, x);
}

// Launch tuning, computed on the device from the level's actual size, so a
// launch whose parent count is only known on the device is tuned the same way.
// Both passes derive the split parameters from the same inputs.
struct Tune {
    unsigned long long n_parents, n_items;
    uint32_t claim_batch;    // chunks claimed per atomic (keeps ~2 claims per warp on big levels)
    uint32_t credit_block;   // output rows reserved per budget atomic; idle credit stays under 1/4 of the level
    uint32_t heavy_thresh;   // candidate slots above which a chunk is split: finer when chunks are few
    uint32_t heavy_piece;    // slots per piece of a split chunk
};

__device__ __forceinline__ Tune make_tune(const ExpandParams& P, bool main_pass) {
    Tune t;
    if (P.n_parents_dev) {
        t.n_parents = *(const volatile unsigned long long*)P.n_parents_dev;
        t.n_items = (t.n_parents + 31) / 32;
    } else {
        t.n_parents = P.n_parents;
        t.n_items = P.n_items;
    }
    const unsigned long long all_warps = P.max_warps ? P.max_warps : 1;
    if (main_pass) {
        // roots cost the same per chunk, so they can be claimed in big batches;
        // deeper chunks vary, so batches stay small there to keep warps balanced
        const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x / 32);
        const unsigned long long per_warp = t.n_items / warps + 1;
        const unsigned long long b = per_warp / (P.pin ? 16 : 2);
        t.claim_batch = (uint32_t)(b < 1 ? 1 : (b > 8 ? 8 : b));
    } else {
        t.claim_batch = 1;
    }
    const unsigned long long cb = P.ocap / (4 * all_warps);
    t.credit_block = (uint32_t)(cb < 1024 ? cb : 1024);
    t.heavy_thresh = t.n_items >= 4 * all_warps ? 4096u : (t.n_items >= all_warps ? 1024u : 256u);
    t.heavy_piece = t.heavy_thresh / 2;
    return t;
}

__device__ __forceinline__ uint32_t item_chunk(const ExpandParams& P, unsigned long long item) {
    return item < P.ndef_in ? P.def_in[(P.def_in_pos + item) % P.def_cap]
                            : (uint32_t)(P.fresh_base + (item - P.ndef_in));
}

__device__ __forceinline__ void defer_chunk(const ExpandParams& P, uint32_t chunk) {
    const unsigned idx = atomicAdd(&P.ctl->ndef, 1u);
    const uint32_t room = P.def_room ? P.def_room : P.def_cap;
    if (idx < room) P.def_out[(P.def_out_pos + idx) % P.def_cap] = chunk;
    else atomicOr(&P.ctl->error, 1u);
}

// Does driver value x (position t of parent j's driver list dj) survive?
// Membership in the other lists first (most candidates fail there), then
// injectivity against the parent's row in shared memory (rarely fails).
template <bool DUPS>
__device__ __forceinline__ bool slot_check(const ExpandParams& P, uint32_t x, uint32_t t, uint32_t j, uint32_t dj,
                                           const uint4& ds, const uint4* segs_s, const uint32_t* rows_s,
                                           uint32_t k, uint32_t d, const uint32_t* stage) {
    bool ok = true;
    uint32_t need = 1;
    if (DUPS) need = seg_rank(ds, t, x, P.nbr) + 1;
    for (uint32_t i = 0; i < k && ok; i++) {
        if (i == dj) continue;
        ok = dev::seg_has_st(segs_s[i * 32 + j], x, need, P.nbr, P.bm, P.bm_words, stage);
    }
    for (uint32_t c = 0; c < d && ok; c++) ok = rows_s[c * 32 + j] != x;
    return ok;
}

// Per-warp shared memory.
struct WarpMem {
    uint32_t* rows_s;   // [d][32] parent rows of the current chunk, column-major
    uint4* segs_s;      // [k][32] segment records
    uint32_t* excl_s;   // [32] exclusive prefix of driver lengths
    uint32_t* drv_s;    // [32] driver list of each parent
    uint32_t* stp;      // [kStage] staged survivors: parent index in the level
    uint32_t* stx;      // [kStage] staged survivors: new vertex
    uint64_t* mbar;     // completion barrier of the list stage's bulk copies
    uint32_t* stage;    // [stage_words] membership lists copied in by TMA (optional)
};

__host__ __device__ constexpr uint32_t per_warp_bytes(uint32_t d, uint32_t k, uint32_t stage_words = 0) {
    return 128 * d + 512 * k + 256 + 8 * kStage + 4 * stage_words;
}

__device__ __forceinline__ WarpMem warp_mem(unsigned char* smem_raw, uint32_t warp, uint32_t d, uint32_t k,
                                            uint32_t stage_words, uint64_t* mbar_s) {
    unsigned char* ws = smem_raw + warp * per_warp_bytes(d, k, stage_words);
    WarpMem m;
    m.rows_s = (uint32_t*)ws;
    m.segs_s = (uint4*)(ws + 128 * d);
    m.excl_s = (uint32_t*)(ws + 128 * d + 512 * k);
    m.drv_s = m.excl_s + 32;
    m.stp = (uint32_t*)(ws + 128 * d + 512 * k + 256);
    m.stx = m.stp + kStage;
    m.mbar = mbar_s + warp;
    m.stage = (uint32_t*)(ws + 128 * d + 512 * k + 256 + 8 * kStage);
    return m;
}

// Membership lists longer than this many words are not staged.
constexpr uint32_t kStageMaxList = 2048;
// Bound on the polls of one stage's completion barrier.
constexpr uint32_t kStageSpinLimit = 1u << 22;

// Stage the membership lists of the loaded chunk: every lane's non-driver
// lists of 4..kStageMaxList entries without a bitmap that its parent's
// candidates probe often enough for the copy to pay (the list-length ratio
// rule of dev::stage_worth) are copied into the warp's stage with TMA bulk copies
// (lanes in order while the stage has room) and their records in segs_s are
// pointed at the stage.  Lane 0 arms the barrier with the byte count, every
// lane issues its own copies, and the warp waits for the phase, boundedly.
// Returns false (warp-uniform) if the wait ran out; the error bit 2 of the
// level's control block is then raised.
__device__ __forceinline__ bool stage_lists(const ExpandParams& P, const WarpMem& m, uint32_t lane, uint32_t k,
                                            uint32_t drv, uint32_t n, bool valid, uint32_t& phase) {
    uint32_t want = 0;
    if (valid && k >= 2 && n >= 2) {
        for (uint32_t i = 0; i < k; i++) {
            if (i == drv) continue;
            const uint4 r = m.segs_s[i * 32 + lane];
            if (dev::stage_worth(r, n, kStageMaxList)) want += (r.x + 3) & ~3u;
        }
    }
    uint32_t incl = want;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if ((int)lane >= o) incl += t;
    }
    const bool fits = want && incl <= P.stage_words;
    uint32_t bytes = fits ? want * 4 : 0;
#pragma unroll
    for (int o = 16; o; o >>= 1) bytes += __shfl_xor_sync(kFull, bytes, o);
    if (!bytes) return true;
    // earlier generic reads of the stage come before the copies overwrite it
    dev::fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) dev::mbar_arrive_expect_tx(m.mbar, bytes);
    __syncwarp();
    if (fits) {
        uint32_t off = incl - want;
        for (uint32_t i = 0; i < k; i++) {
            if (i == drv) continue;
            uint4 r = m.segs_s[i * 32 + lane];
            if (dev::stage_worth(r, n, kStageMaxList)) {
                const uint32_t words = (r.x + 3) & ~3u;
                dev::bulk_copy_g2s(m.stage + off, P.nbr + (uint64_t)r.y * 4, words * 4, m.mbar);
                r.y = dev::kStagedMark | off;
                m.segs_s[i * 32 + lane] = r;
                off += words;
            }
        }
    }
    bool ok = false;
    for (uint32_t spin = 0; spin < kStageSpinLimit && !ok; spin++) ok = dev::mbar_try_wait(m.mbar, phase);
    phase ^= 1u;
    ok = __all_sync(kFull, ok);
    if (!ok && lane == 0) atomicOr(&P.ctl->error, 2u);
    __syncwarp();
    return ok;
}

// Column c of parent p of the level being expanded.
template <bool ROOTS>
__device__ __forceinline__ uint32_t parent_col(const ExpandParams& P, uint32_t c, uint32_t p) {
    if (ROOTS) return P.root_list ? __ldg(P.root_list + p) : P.root_begin + p;
    return __ldg(P.pin + c * P.pstride + p);
}

// Column c of staged parent p: from the warp's copy of chunk `cur` in shared
// memory when p belongs to it (most survivors do), else from the level.
template <bool ROOTS>
__device__ __forceinline__ uint32_t staged_col(const ExpandParams& P, const WarpMem& m, uint32_t c, uint32_t p,
                                               uint32_t cur) {
    if ((p >> 5) == cur) return m.rows_s[c * 32 + (p & 31)];
    return parent_col<ROOTS>(P, c, p);
}

// Write the staged survivors with one atomic: column by column into the next
// level (SoA), or row-major into the table; every store is coalesced.  `cur`
// is the chunk whose rows the warp holds in shared memory.
template <int MODE, bool ROOTS>
__device__ __forceinline__ void flush_stage(const ExpandParams& P, const WarpMem& m, uint32_t nst, uint32_t lane,
                                            uint32_t d, const uint8_t* col_depth_s, uint32_t cur) {
    unsigned long long pos0 = 0;
    if (lane == 0)
        pos0 = atomicAdd(MODE == kModeMid ? &P.ctl->produced : &P.tot->table_pos, (unsigned long long)nst);
    pos0 = __shfl_sync(kFull, pos0, 0);
    if (MODE == kModeMid) {
        for (uint32_t c = 0; c < d; c++) {
            uint32_t* col = P.pout + c * P.ocap + pos0;
            for (uint32_t i = lane; i < nst; i += 32) col[i] = staged_col<ROOTS>(P, m, c, m.stp[i], cur);
        }
        uint32_t* col = P.pout + d * P.ocap + pos0;
        for (uint32_t i = lane; i < nst; i += 32) col[i] = m.stx[i];
    } else {
        // one row per lane; the warp's rows are contiguous, so the vector
        // stores of a round cover one block of 32 * 4q bytes
        const uint32_t q = P.plan.q;
        if (pos0 >= P.table_cap) return;
        const uint64_t room = P.table_cap - pos0;
        const uint32_t rows = nst < room ? nst : (uint32_t)room;
        uint32_t* out = P.table + pos0 * q;
        for (uint32_t r = lane; r < rows; r += 32) {
            const uint32_t p = m.stp[r], x = m.stx[r];
            uint32_t* o = out + (uint64_t)r * q;
            if (P.table_vec4) {
                for (uint32_t c = 0; c < q; c += 4) {
                    uint4 v;
                    uint32_t dep = col_depth_s[c];
                    v.x = dep < d ? staged_col<ROOTS>(P, m, dep, p, cur) : x;
                    dep = col_depth_s[c + 1];
                    v.y = dep < d ? staged_col<ROOTS>(P, m, dep, p, cur) : x;
                    dep = col_depth_s[c + 2];
                    v.z = dep < d ? staged_col<ROOTS>(P, m, dep, p, cur) : x;
                    dep = col_depth_s[c + 3];
                    v.w = dep < d ? staged_col<ROOTS>(P, m, dep, p, cur) : x;
                    *(uint4*)(o + c) = v;
                }
            } else {
                for (uint32_t c = 0; c < q; c++) {
                    const uint32_t dep = col_depth_s[c];
                    o[c] = dep < d ? staged_col<ROOTS>(P, m, dep, p, cur) : x;
                }
            }
        }
    }
}

// Load the 32 parents of `chunk`, look up their k lists (independent 16-byte
// loads), pick each parent's shortest list as its driver and prefix-sum the
// driver lengths.  Returns the chunk's candidate slots (warp-uniform).
template <bool ROOTS>
__device__ __forceinline__ uint32_t load_chunk(const ExpandParams& P, const WarpMem& m, uint32_t chunk, uint32_t lane,
                                               uint32_t d, uint32_t k, uint32_t rb, unsigned long long n_parents,
                                               bool& valid, unsigned long long& words, uint32_t& phase,
                                               bool& stage_ok) {
    const uint64_t p = (uint64_t)chunk * 32 + lane;
    valid = p < n_parents;
    if (ROOTS) {
        m.rows_s[lane] = !P.root_list ? P.root_begin + (uint32_t)p : valid ? __ldg(P.root_list + p) : 0u;
    } else {
        for (uint32_t c = 0; c < d; c++) m.rows_s[c * 32 + lane] = valid ? P.pin[c * P.pstride + p] : 0u;
    }
    uint32_t n = 0, drv = 0;
    words = 0;
    if (valid) {
        uint32_t best = 0xffffffffu;
        for (uint32_t i = 0; i < k; i++) {
            const uint32_t anc = P.plan.req_anc[rb + i];
            const uint32_t lab = P.plan.req_label[rb + i];
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
    }
    stage_ok = true;
    if (P.stage_words && k >= 2) stage_ok = stage_lists(P, m, lane, k, drv, n, valid, phase);
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if ((int)lane >= o) incl += t;
    }
    m.excl_s[lane] = incl - n;
    m.drv_s[lane] = drv;
    __syncwarp();
    return __shfl_sync(kFull, incl, 31);
}

// Work counters of the last depth under pre-count (lane-private): the
// survivors stand for that depth's parents, one lookup each, and their
// lists' lengths for its list words.
struct PreAcc {
    unsigned long long parents = 0, words = 0;
};

// Adds a warp's pre-count work counters to the next depth's control block,
// so the last depth reports the same work as when it is launched.
__device__ __forceinline__ void flush_pre(const ExpandParams& P, PreAcc& pre, uint32_t lane) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        pre.parents += __shfl_down_sync(kFull, pre.parents, o);
        pre.words += __shfl_down_sync(kFull, pre.words, o);
    }
    if (lane == 0 && pre.parents) {
        LaunchCtl* next = P.ctl + 1;
        atomicAdd(&next->parents, pre.parents);
        atomicAdd(&next->lookups, pre.parents);
        atomicAdd(&next->list_words, pre.words);
    }
}

// Evaluate slots [begin, end) of the loaded chunk: kSlots slots per lane per
// round with all their driver loads in flight; survivors go to the stage,
// which is flushed whenever it cannot take another round.
template <int MODE, bool ROOTS, bool DUPS>
__device__ __forceinline__ void process_slots(const ExpandParams& P, const WarpMem& m, uint32_t chunk,
                                              uint32_t begin, uint32_t end, uint32_t lane, uint32_t d, uint32_t k,
                                              const uint8_t* col_depth_s, uint32_t& nst,
                                              unsigned long long& n_count, PreAcc& pre) {
    const uint32_t pbase = chunk * 32;
    unsigned long long lane_count = 0;   // pre-count: this lane's counts, summed over the warp at the end
    for (uint32_t base = begin; base < end; base += 32 * kSlots) {
        uint32_t j[kSlots], t[kSlots], x[kSlots];
        bool ok[kSlots];
        // every driver load of the round is issued before any check
#pragma unroll
        for (uint32_t u = 0; u < kSlots; u++) {
            const uint32_t s = base + 32 * u + lane;
            j[u] = t[u] = x[u] = 0;
            ok[u] = s < end;
            if (ok[u]) {
                slot_locate(s, m.excl_s, j[u], t[u]);
                x[u] = seg_at(m.segs_s[m.drv_s[j[u]] * 32 + j[u]], t[u], P.nbr);
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kSlots; u++) {
            if (ok[u]) {
                const uint32_t dj = m.drv_s[j[u]];
                ok[u] = slot_check<DUPS>(P, x[u], t[u], j[u], dj, m.segs_s[dj * 32 + j[u]], m.segs_s, m.rows_s, k, d,
                                         m.stage);
            }
        }
        if (MODE == kModeLastCount && !DUPS && P.pre_count) {
            // Pre-count: each survivor's extensions at the last depth (one back
            // edge: ancestor anc, label lab) are the entries of that list minus
            // the row's vertices found in it; the survivor is never stored.
            const uint32_t rb = P.plan.req_begin[d + 1];
            const uint32_t anc = P.plan.req_anc[rb];
            const uint4* segl = P.seg + (uint64_t)P.plan.req_label[rb] * P.V;
#pragma unroll
            for (uint32_t u = 0; u < kSlots; u++) {
                uint32_t c = 0;
                if (ok[u]) {
                    const uint4 sg = ldg4(segl + (anc == d ? x[u] : m.rows_s[anc * 32 + j[u]]));
                    c = sg.x - dev::count_members(sg, m.rows_s, j[u], d, x[u], P.self_loops || anc != d, P.nbr,
                                                  P.bm, P.bm_words);
                    pre.parents += 1;
                    pre.words += sg.x;
                }
                lane_count += c;
            }
            continue;
        }
        const unsigned lt = (1u << lane) - 1u;
#pragma unroll
        for (uint32_t u = 0; u < kSlots; u++) {
            const unsigned b = __ballot_sync(kFull, ok[u]);
            if (MODE == kModeLastCount) {
                n_count += __popc(b);
                continue;
            }
            if (ok[u]) {
                const uint32_t q = nst + __popc(b & lt);
                m.stp[q] = pbase + j[u];
                m.stx[q] = x[u];
            }
            nst += __popc(b);
        }
        if (MODE == kModeLastCount) continue;
        if (nst > kStage - 32 * kSlots) {
            __syncwarp();
            flush_stage<MODE, ROOTS>(P, m, nst, lane, d, col_depth_s, chunk);
            nst = 0;
        }
        __syncwarp();
    }
    if (MODE == kModeLastCount && !DUPS && P.pre_count) {
#pragma unroll
        for (int o = 16; o; o >>= 1) lane_count += __shfl_xor_sync(kFull, lane_count, o);
        n_count += lane_count;
    }
}

// Work limit of a last level (warp-uniform result): lane 0 adds the warp's
// recent count to the total, compares the total (or the table rows reserved)
// with the limit and raises the limit flag.  Checked once per chunk or piece,
// so a warp overshoots by at most one chunk's work.
template <int MODE>
__device__ __forceinline__ bool over_limit(const ExpandParams& P, uint32_t lane, unsigned long long n_count,
                                           unsigned long long& n_flushed) {
    int over = 0;
    if (lane == 0) {
        unsigned long long seen;
        if (MODE == kModeLastCount) {
            seen = *(volatile unsigned long long*)&P.tot->count;
            if (n_count - n_flushed >= 4096) {
                seen = atomicAdd(&P.tot->count, n_count - n_flushed) + (n_count - n_flushed);
                n_flushed = n_count;
            }
        } else {
            seen = *(volatile unsigned long long*)&P.tot->table_pos;
        }
        if (seen > P.work_limit) {
            over = 1;
            atomicOr(&P.tot->error, kLimitFlag);
        }
    }
    return __shfl_sync(kFull, over, 0) != 0;
}

// Main pass: warps claim batches of chunks; long candidate ranges are
// published to the heavy list instead of being walked by one warp.
template <int MODE, bool ROOTS, bool DUPS>
__device__ __forceinline__ void expand_main(const ExpandParams& P, unsigned char* smem_raw,
                                            const uint8_t* col_depth_s, uint64_t* mbar_s, uint32_t& phase) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t d = P.depth;
    const uint32_t k = P.plan.nreq[d];
    const uint32_t rb = P.plan.req_begin[d];
    const uint32_t sw = k >= 2 ? P.stage_words : 0;   // only levels with membership tests stage lists
    const WarpMem m = warp_mem(smem_raw, threadIdx.x >> 5, d, k, sw, mbar_s);
    const Tune T = make_tune(P, true);

    unsigned long long n_count = 0, n_lookups = 0, n_words = 0, n_parents = 0;
    unsigned long long n_flushed = 0;  // part of n_count already added to tot->count (lane 0)
    PreAcc pre;
    uint32_t last_chunk = 0xffffffffu;   // chunk whose rows are in m.rows_s
    unsigned long long credit = 0;   // level budget held by this warp (lane 0)
    uint32_t nst = 0;
    bool done = false;
    while (!done) {
        unsigned long long first = 0;
        if (lane == 0) first = atomicAdd(&P.ctl->claim, (unsigned long long)T.claim_batch);
        first = __shfl_sync(kFull, first, 0);
        if (first >= T.n_items) break;
        const unsigned long long last =
            first + T.claim_batch < T.n_items ? first + T.claim_batch : T.n_items;
        for (unsigned long long item = first; item < last; item++) {
            const uint32_t chunk = item_chunk(P, item);
            if (MODE != kModeMid && P.work_limit && over_limit<MODE>(P, lane, n_count, n_flushed)) {
                done = true;
                break;
            }
            if (MODE == kModeMid) {
                // one lane reads the flag and broadcasts it, so the warp never splits
                int stop = 0;
                if (lane == 0) stop = *(volatile unsigned int*)&P.ctl->stop ? 1 : 0;
                stop = __shfl_sync(kFull, stop, 0);
                if (stop) {
                    if (lane == 0)
                        for (unsigned long long it = item; it < last; it++) defer_chunk(P, item_chunk(P, it));
                    done = true;
                    break;
                }
            }
            bool valid, stage_ok;
            unsigned long long w;
            const uint32_t total = load_chunk<ROOTS>(P, m, chunk, lane, d, k, rb, T.n_parents, valid, w, phase,
                                                     stage_ok);
            last_chunk = chunk;
            if (!stage_ok) {
                done = true;
                break;
            }
            if (MODE == kModeLastCount && !DUPS && k == 1 && !P.pre_count) {
                // Count rule: with one requirement every list entry extends the
                // parent except the parent's own vertices, so each lane counts
                // its parent's extensions as the list length minus the row's
                // vertices found in the list; no candidate is enumerated.
                unsigned long long c = 0;
                if (valid) {
                    const uint4 sg = m.segs_s[lane];
                    c = sg.x - dev::count_members(sg, m.rows_s, lane, d, 0u, false, P.nbr, P.bm, P.bm_words);
                    n_lookups += k;
                    n_words += w;
                    n_parents += 1;
                }
#pragma unroll
                for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
                n_count += c;
                continue;
            }
            if (MODE == kModeMid && total) {
                int ok = 1;
                if (lane == 0) {
                    if (total > credit) {
                        const unsigned long long need = max((unsigned long long)total, (unsigned long long)T.credit_block);
                        const unsigned long long old = atomicAdd(&P.ctl->budget, need);
                        if (old + need > P.ocap) {
                            ok = 0;
                            atomicExch(&P.ctl->stop, 1u);
                            for (unsigned long long it = item; it < last; it++) defer_chunk(P, item_chunk(P, it));
                        } else {
                            credit += need;
                        }
                    }
                    if (ok) credit -= total;
                }
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
            if (total > T.heavy_thresh) {
                // Publish: one packed atomic reserves the entry index and its
                // piece range, so entries are ordered by first piece.  The room
                // check is conservative: at most max_warps publishers are past it.
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
            process_slots<MODE, ROOTS, DUPS>(P, m, chunk, 0, total, lane, d, k, col_depth_s, nst, n_count, pre);
        }
    }
    if (MODE != kModeLastCount && nst) flush_stage<MODE, ROOTS>(P, m, nst, lane, d, col_depth_s, last_chunk);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        n_lookups += __shfl_down_sync(kFull, n_lookups, o);
        n_words += __shfl_down_sync(kFull, n_words, o);
        n_parents += __shfl_down_sync(kFull, n_parents, o);
    }
    if (lane == 0) {
        if (n_parents) {
            atomicAdd(&P.ctl->parents, n_parents);
            atomicAdd(&P.ctl->lookups, n_lookups);
            atomicAdd(&P.ctl->list_words, n_words);
        }
        if (MODE == kModeLastCount && n_count > n_flushed) atomicAdd(&P.tot->count, n_count - n_flushed);
    }
    if (MODE == kModeLastCount && !DUPS && P.pre_count) flush_pre(P, pre, lane);
}

// Heavy pass (after the main pass): every warp claims pieces of the published
// chunks, reloads that chunk and walks its piece of the slots -- the warps
// that finished their own chunks take over the work of the hub chunks.  The
// main pass already holds the chunk's output budget and counted its work.
template <int MODE, bool ROOTS, bool DUPS>
__device__ __forceinline__ void expand_heavy(const ExpandParams& P, unsigned char* smem_raw,
                                             const uint8_t* col_depth_s, uint64_t* mbar_s, uint32_t& phase) {
    const unsigned long long h = *(volatile unsigned long long*)&P.ctl->heavy;
    const uint32_t nent = (uint32_t)(h >> 32);
    const uint32_t npieces = (uint32_t)h;
    if (nent == 0) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t d = P.depth;
    const uint32_t k = P.plan.nreq[d];
    const uint32_t rb = P.plan.req_begin[d];
    const uint32_t sw = k >= 2 ? P.stage_words : 0;
    const WarpMem m = warp_mem(smem_raw, threadIdx.x >> 5, d, k, sw, mbar_s);
    const Tune T = make_tune(P, false);
    unsigned long long n_count = 0, n_flushed = 0;
    PreAcc pre;
    uint32_t last_chunk = 0xffffffffu;   // chunk whose rows are in m.rows_s
    uint32_t nst = 0;
    for (;;) {
        if (MODE != kModeMid && P.work_limit && over_limit<MODE>(P, lane, n_count, n_flushed)) break;
        unsigned long long gp = 0;
        if (lane == 0) gp = atomicAdd(&P.ctl->claim2, 1ull);
        gp = __shfl_sync(kFull, gp, 0);
        if (gp >= npieces) break;
        uint32_t lo = 0, hi = nent;      // last entry with piece0 <= gp
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (P.heavy[mid].piece0 <= gp) lo = mid;
            else hi = mid;
        }
        const HeavyEntry e = P.heavy[lo];
        const uint32_t begin = ((uint32_t)gp - e.piece0) * T.heavy_piece;
        const uint32_t end = min(begin + T.heavy_piece, e.total);
        bool valid, stage_ok;
        unsigned long long w;
        load_chunk<ROOTS>(P, m, e.chunk, lane, d, k, rb, T.n_parents, valid, w, phase, stage_ok);
        last_chunk = e.chunk;
        if (!stage_ok) break;
        process_slots<MODE, ROOTS, DUPS>(P, m, e.chunk, begin, end, lane, d, k, col_depth_s, nst, n_count, pre);
    }
    if (MODE != kModeLastCount && nst) flush_stage<MODE, ROOTS>(P, m, nst, lane, d, col_depth_s, last_chunk);
    if (MODE == kModeLastCount && lane == 0 && n_count > n_flushed) atomicAdd(&P.tot->count, n_count - n_flushed);
    if (MODE == kModeLastCount && !DUPS && P.pre_count) flush_pre(P, pre, lane);
}

template <int MODE, bool ROOTS, bool DUPS>
__global__ void __launch_bounds__(kWarps * 32, 6) k_expand(const __grid_constant__ ExpandParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint8_t col_depth_s[kMaxQ];
    __shared__ uint64_t mbar_s[kWarps];
    if (threadIdx.x < (unsigned)kMaxQ) col_depth_s[threadIdx.x] = P.plan.col_depth[threadIdx.x];
    dev::stage_barriers_init(mbar_s);
    uint32_t phase = 0;
    expand_main<MODE, ROOTS, DUPS>(P, smem_raw, col_depth_s, mbar_s, phase);
}

template <int MODE, bool ROOTS, bool DUPS>
__global__ void __launch_bounds__(kWarps * 32, 6) k_expand_heavy(const __grid_constant__ ExpandParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint8_t col_depth_s[kMaxQ];
    __shared__ uint64_t mbar_s[kWarps];
    if (threadIdx.x < (unsigned)kMaxQ) col_depth_s[threadIdx.x] = P.plan.col_depth[threadIdx.x];
    dev::stage_barriers_init(mbar_s);
    uint32_t phase = 0;
    expand_heavy<MODE, ROOTS, DUPS>(P, smem_raw, col_depth_s, mbar_s, phase);
}

// ------------------------------------------------------- persistent engine
//
// One cooperative launch runs every level pass of the match.  A pass of depth
// d is the same main and heavy pass as above, on the work items of the
// depth-d queue: the deferred ring of depth d (chunks pushed back when the
// output level filled) followed by the fresh chunks not yet claimed.  Between
// passes block 0 advances the schedule (dev::sched_advance), so a level whose
// output buffer fills is drained depth first on the device, with no host
// round trip; a level whose chunks are long is cut into pieces that every warp
// takes in the heavy pass.

template <int LAST, bool DUPS>
__device__ __forceinline__ void persist_main(const ExpandParams& P, unsigned char* smem, const uint8_t* cd,
                                             bool roots, bool last, uint64_t* mb, uint32_t& ph) {
    if (last) {
        if (roots) expand_main<LAST, true, DUPS>(P, smem, cd, mb, ph);
        else expand_main<LAST, false, DUPS>(P, smem, cd, mb, ph);
    } else {
        if (roots) expand_main<kModeMid, true, DUPS>(P, smem, cd, mb, ph);
        else expand_main<kModeMid, false, DUPS>(P, smem, cd, mb, ph);
    }
}

template <int LAST, bool DUPS>
__device__ __forceinline__ void persist_heavy(const ExpandParams& P, unsigned char* smem, const uint8_t* cd,
                                              bool roots, bool last, uint64_t* mb, uint32_t& ph) {
    if (last) {
        if (roots) expand_heavy<LAST, true, DUPS>(P, smem, cd, mb, ph);
        else expand_heavy<LAST, false, DUPS>(P, smem, cd, mb, ph);
    } else {
        if (roots) expand_heavy<kModeMid, true, DUPS>(P, smem, cd, mb, ph);
        else expand_heavy<kModeMid, false, DUPS>(P, smem, cd, mb, ph);
    }
}

template <int LAST, bool DUPS>
__global__ void __launch_bounds__(kWarps * 32, 5) k_persist(const __grid_constant__ ExpandParams P0,
                                                            const __grid_constant__ PersistArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) ExpandParams P;          // level fields change per pass
    __shared__ uint8_t col_depth_s[kMaxQ];
    __shared__ unsigned flag_s, cur_s;
    __shared__ uint64_t mbar_s[kWarps];
    SchedState* S = A.sched;
    {
        const uint32_t* src = (const uint32_t*)&P0;
        uint32_t* dst = (uint32_t*)&P;
        for (uint32_t i = threadIdx.x; i < sizeof(ExpandParams) / 4; i += blockDim.x) dst[i] = src[i];
    }
    if (threadIdx.x < (unsigned)kMaxQ) col_depth_s[threadIdx.x] = P0.plan.col_depth[threadIdx.x];
    dev::stage_barriers_init(mbar_s);
    uint32_t phase = 0;       // of this warp's stage barrier, carried across passes
    const uint32_t q = P0.plan.q;
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
                P.pin = d == 1 ? nullptr : A.levels[d];
                P.pout = d + 1 + P0.pre_count < q ? A.levels[d + 1] : nullptr;
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
        const bool roots = d == 1, last = d + 1 + P0.pre_count == q;
        persist_main<LAST, DUPS>(P, smem_raw, col_depth_s, roots, last, mbar_s, phase);
        if (!dev::grid_barrier(S, first && A.hold_first_barrier && blockIdx.x == 0, &flag_s)) break;
        first = false;
        persist_heavy<LAST, DUPS>(P, smem_raw, col_depth_s, roots, last, mbar_s, phase);
        if (!dev::grid_barrier(S, false, &flag_s)) break;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const bool limit_hit = P.work_limit && (*(volatile unsigned*)&P.tot->error & kLimitFlag);
            dev::sched_advance(S, P0.ctl, d, !last, P.n_items, P.ndef_in, P.def_room, limit_hit);
        }
        if (!dev::grid_barrier(S, false, &flag_s)) break;
    }
}

template <int MODE, bool ROOTS, bool DUPS>
void* kernel_ptr(bool heavy) {
    return heavy ? (void*)&k_expand_heavy<MODE, ROOTS, DUPS> : (void*)&k_expand<MODE, ROOTS, DUPS>;
}

void* pick(int mode, bool roots, bool dups, bool heavy) {
#define FM_PICK(M)                                                                                     \
    if (mode == M) {                                                                                   \
        if (roots) return dups ? kernel_ptr<M, true, true>(heavy) : kernel_ptr<M, true, false>(heavy); \
        return dups ? kernel_ptr<M, false, true>(heavy) : kernel_ptr<M, false, false>(heavy);          \
    }
    FM_PICK(kModeMid)
    FM_PICK(kModeLastTable)
    FM_PICK(kModeLastCount)
#undef FM_PICK
    return nullptr;
}

void* persist_ptr(int last_mode, bool dups) {
    if (last_mode == kModeLastTable) return dups ? (void*)&k_persist<kModeLastTable, true> : (void*)&k_persist<kModeLastTable, false>;
    return dups ? (void*)&k_persist<kModeLastCount, true> : (void*)&k_persist<kModeLastCount, false>;
}

}  // namespace

namespace {
// Initial schedule: every pass starts at depth 1 on n_roots root rows.  A
// kernel rather than a host copy, so a captured CUDA graph replays it.
__global__ void k_sched_init(SchedState* S, unsigned q, unsigned long long n_roots, unsigned long long work_limit,
                             unsigned long long wait_ns) {
    unsigned* w = (unsigned*)S;
    for (unsigned i = threadIdx.x; i < sizeof(SchedState) / 4; i += blockDim.x) w[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        S->cur = 1;
        S->q = q;
        S->work_limit = work_limit;
        S->wait_limit_ns = wait_ns;
        S->lv[1].n_parents = n_roots;
    }
}
}  // namespace

cudaError_t launch_sched_init(SchedState* S, unsigned q, unsigned long long n_roots, unsigned long long work_limit,
                              unsigned long long wait_ns, cudaStream_t s) {
    k_sched_init<<<1, 128, 0, s>>>(S, q, n_roots, work_limit, wait_ns);
    return cudaGetLastError();
}

size_t persist_smem_bytes(const DevPlan& plan, const uint32_t* nreq_depth, uint32_t stage_words) {
    size_t best = 0;
    for (uint32_t d = 1; d < plan.q; d++)
        best = std::max<size_t>(best, per_warp_bytes(d, nreq_depth[d], nreq_depth[d] >= 2 ? stage_words : 0));
    return best * kWarps;
}

int persist_blocks_per_sm(int last_mode, bool dups, size_t smem) {
    void* f = persist_ptr(last_mode, dups);
    allow_dynamic_smem(f);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, kWarps * 32, smem) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    return n;
}

cudaError_t launch_persist(const ExpandParams& p, const PersistArgs& a, int last_mode, bool dups, int grid,
                           size_t smem, cudaStream_t s) {
    ExpandParams q = p;
    q.max_warps = (uint32_t)grid * kWarps;
    q.n_parents_dev = nullptr;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kWarps * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {(void*)&q, (void*)&a};
    return cudaLaunchKernelExC(&cfg, persist_ptr(last_mode, dups), args);
}

size_t expand_smem_bytes(uint32_t depth, uint32_t nreq, int warps, uint32_t stage_words) {
    return (size_t)warps * per_warp_bytes(depth, nreq, stage_words);
}

void allow_dynamic_smem(const void* f) {
    // Raised once per (device, kernel) to the opt-in maximum: a per-launch
    // value would race between host threads launching with different sizes.
    static std::mutex mu;
    static std::set<std::pair<int, const void*>> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (!done.insert({dev, f}).second) return;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, f) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    // static shared memory counts against the same opt-in limit
    const int dyn = optin - (int)fa.sharedSizeBytes;
    if (dyn > 0 && cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
        cudaGetLastError();   // the launch reports a size it cannot take
}

int expand_blocks_per_sm(int mode, bool roots, bool dups, size_t smem, int block) {
    void* f = pick(mode, roots, dups, false);
    allow_dynamic_smem(f);
    allow_dynamic_smem(pick(mode, roots, dups, true));
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, block, smem) != cudaSuccess || n < 1) n = 1;
    return n;
}

cudaError_t launch_expand(const ExpandParams& p, int mode, bool roots, bool dups, int grid, int heavy_grid,
                          int block, size_t smem, cudaStream_t s) {
    void* f = pick(mode, roots, dups, false);
    void* fh = pick(mode, roots, dups, true);
    if (!f || !fh) return cudaErrorInvalidValue;
    ExpandParams q = p;
    // both passes tune themselves on the device (make_tune) from the level size
    // and from max_warps, the warps of the heavy pass
    q.max_warps = (uint32_t)heavy_grid * (uint32_t)(block / 32);
    void* args[] = {(void*)&q};
    cudaError_t e = cudaLaunchKernel(f, dim3(grid), dim3(block), args, smem, s);
    if (e != cudaSuccess) return e;
    // the heavy pass always gets a full grid: a few heavy chunks can hold most of the work
    return cudaLaunchKernel(fh, dim3(heavy_grid), dim3(block), args, smem, s);
}

}  // namespace fm
