// fm_device.cuh -- device helpers shared by the level-expansion kernels.
#pragma once

#include "fm_internal.h"

namespace fm {
namespace dev {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ uint4 ldg4(const uint4* p) { return __ldg(p); }

// Element t of a (label, vertex) list given its segment record.
__device__ __forceinline__ uint32_t seg_at(const uint4& s, uint32_t t, const uint32_t* __restrict__ nbr) {
    if (s.x <= 3) return t == 0 ? s.y : (t == 1 ? s.z : s.w);
    return __ldg(nbr + (uint64_t)s.y * 4 + t);
}

// lower_bound of x in a[0, n)
__device__ __forceinline__ uint32_t lower_bound_g(const uint32_t* __restrict__ a, uint32_t n, uint32_t x) {
    uint32_t lo = 0;
    while (n > 0) {
        const uint32_t half = n >> 1;
        if (__ldg(a + lo + half) < x) {
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

// Does the list hold at least `need` copies of x?  Lists with a bitmap
// (graphs without duplicate e-lines only, so need == 1) answer with one load.
__device__ __forceinline__ bool seg_has(const uint4& s, uint32_t x, uint32_t need, const uint32_t* __restrict__ nbr,
                                        const uint32_t* __restrict__ bm, uint32_t bm_words) {
    if (s.x <= 3) {
        // an empty list's record is all zero; in a non-empty one the unused
        // inline slots hold kNoVertex, which no vertex id equals
        if (s.x == 0) return false;
        const uint32_t c = (s.y == x) + (s.z == x) + (s.w == x);
        return c >= need;
    }
    if (x > s.w) return false;
    if (s.z & kBitmapMark) {
        const uint32_t* b = bm + (uint64_t)(s.z & ~kBitmapMark) * bm_words;
        return (__ldg(b + (x >> 5)) >> (x & 31)) & 1u;
    }
    if (x < s.z) return false;
    const uint32_t* a = nbr + (uint64_t)s.y * 4;
    const uint32_t pos = lower_bound_g(a, s.x, x) + need - 1;
    return pos < s.x && __ldg(a + pos) == x;
}

// How many of the row's vertices (column-major rows_s[c*32 + j], c < n_row)
// and, with `extra`, the value x, are in the list of record s.  Graphs
// without duplicate e-lines only (a value is in a list at most once); the
// values are distinct (an injective row plus a new vertex).  Used by the
// count rule, where every one of these membership tests is needed: inline
// lists compare in registers, bitmap lists take one independent load per
// value, and long lists are searched for four values in lockstep
// (branch-free search for the last entry <= value: every step issues its
// four loads together, so the searches overlap instead of running one after
// another).
__device__ __forceinline__ uint32_t count_members(const uint4& s, const uint32_t* rows_s, uint32_t j, uint32_t n_row,
                                                  uint32_t x, bool extra, const uint32_t* __restrict__ nbr,
                                                  const uint32_t* __restrict__ bm, uint32_t bm_words) {
    const uint32_t n = n_row + (extra ? 1u : 0u);
    uint32_t found = 0;
    if (s.x == 0) return 0;
    if (s.x <= 3) {
        // s.x >= 1 here; unused inline slots hold kNoVertex, which no vertex id equals
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t v = i < n_row ? rows_s[i * 32 + j] : x;
            found += (s.y == v) + (s.z == v) + (s.w == v);
        }
        return found;
    }
    if (s.z & kBitmapMark) {
        const uint32_t* b = bm + (uint64_t)(s.z & ~kBitmapMark) * bm_words;
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t v = i < n_row ? rows_s[i * 32 + j] : x;
            found += v <= s.w ? (__ldg(b + (v >> 5)) >> (v & 31)) & 1u : 0u;
        }
        return found;
    }
    const uint32_t* a = nbr + (uint64_t)s.y * 4;
    for (uint32_t g = 0; g < n; g += 4) {
        uint32_t key[4], base[4];
        bool act[4];
#pragma unroll
        for (uint32_t u = 0; u < 4; u++) {
            const uint32_t i = g + u;
            key[u] = i < n_row ? rows_s[i * 32 + j] : x;
            act[u] = i < n && key[u] >= s.z && key[u] <= s.w;
            base[u] = 0;
        }
        uint32_t len = s.x;
        while (len > 1) {
            const uint32_t half = len >> 1;
#pragma unroll
            for (uint32_t u = 0; u < 4; u++)
                if (act[u] && __ldg(a + base[u] + half) <= key[u]) base[u] += half;
            len -= half;
        }
#pragma unroll
        for (uint32_t u = 0; u < 4; u++) found += (act[u] && __ldg(a + base[u]) == key[u]) ? 1u : 0u;
    }
    return found;
}

// ------------------------------------------------- staged membership lists
//
// A list tested for membership by many candidates of a chunk is copied once
// into the warp's shared-memory stage with a TMA bulk copy and searched there.
// Its record then holds the stage offset in the `off16` field with kStagedMark
// set (global offsets stay below 2^31 sixteen-byte units).
constexpr uint32_t kStagedMark = 0x80000000u;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes generic-proxy accesses to shared memory (and an mbarrier init)
// visible to the async proxy before later bulk copies.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Makes mbarrier initialisations visible to the async proxy (the bulk
// copies' complete_tx) before any copy refers to them.
__device__ __forceinline__ void fence_mbarrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One completion barrier per warp for the list stage, in static shared memory
// at a fixed place for the whole launch: initialised once (arrival count 1:
// lane 0 arms each phase), fenced, then the block synchronises.
__device__ __forceinline__ void stage_barriers_init(uint64_t* mbar_s) {
    if ((threadIdx.x & 31) == 0) mbar_init(&mbar_s[threadIdx.x >> 5], 1);
    fence_mbarrier_init();
    __syncthreads();
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// One TMA bulk copy global -> shared (16-byte aligned ends, size a multiple
// of 16 bytes), completing on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// lower_bound of x in a[0, n) in shared memory
__device__ __forceinline__ uint32_t lower_bound_s(const uint32_t* a, uint32_t n, uint32_t x) {
    uint32_t lo = 0;
    while (n > 0) {
        const uint32_t half = n >> 1;
        if (a[lo + half] < x) {
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

// Intersection method of one membership list, chosen per parent by the
// list-length ratio: a list of n entries probed by the m candidates of the
// parent's driver list is copied into the warp's shared-memory stage (a TMA
// bulk copy, then binary searches in shared memory) when the candidates'
// searches in global memory, about m * ceil(log2 n) dependent loads, outweigh
// copying its n / 32 128-byte lines; with a more skewed ratio each candidate
// searches the list in global memory.  Inline lists (<= 3 entries) compare in
// registers and bitmap lists take one load, so neither is staged.
__device__ __forceinline__ bool stage_worth(const uint4& r, uint32_t m, uint32_t max_list) {
    if (r.x <= 3 || r.x > max_list || (r.z & kBitmapMark)) return false;
    const uint32_t lg = 32u - __clz(r.x - 1u);
    return (unsigned long long)m * 32u * lg >= r.x;
}

// seg_has for records that may point into the warp's stage.
__device__ __forceinline__ bool seg_has_st(const uint4& s, uint32_t x, uint32_t need, const uint32_t* __restrict__ nbr,
                                           const uint32_t* __restrict__ bm, uint32_t bm_words, const uint32_t* stage) {
    if (s.x > 3 && (s.y & kStagedMark)) {
        if (x > s.w || x < s.z) return false;
        const uint32_t* a = stage + (s.y & ~kStagedMark);
        const uint32_t pos = lower_bound_s(a, s.x, x) + need - 1;
        return pos < s.x && a[pos] == x;
    }
    return seg_has(s, x, need, nbr, bm, bm_words);
}

// Reorder one parent's records (column `lane` of recs): the driver first, the
// other lists shortest first, so a candidate meets the most selective
// membership test first and most rejections take one test.  Returns the
// driver's new index (0).  Membership does not depend on the order.
__device__ __forceinline__ uint32_t order_lists(uint4* recs, uint32_t lane, uint32_t k, uint32_t drv) {
    if (drv != 0) {
        const uint4 t = recs[lane];
        recs[lane] = recs[drv * 32 + lane];
        recs[drv * 32 + lane] = t;
    }
    for (uint32_t i = 2; i < k; i++) {
        const uint4 key = recs[i * 32 + lane];
        uint32_t j = i;
        while (j > 1 && recs[(j - 1) * 32 + lane].x > key.x) {
            recs[j * 32 + lane] = recs[(j - 1) * 32 + lane];
            j--;
        }
        recs[j * 32 + lane] = key;
    }
    return 0;
}

// Slot s of a chunk belongs to parent j (the last j with excl[j] <= s), at
// position t of that parent's driver list.
__device__ __forceinline__ void slot_locate(uint32_t s, const uint32_t* excl_s, uint32_t& j, uint32_t& t) {
    j = 0;
#pragma unroll
    for (uint32_t step = 16; step; step >>= 1)
        if (excl_s[j + step] <= s) j += step;
    t = s - excl_s[j];
}

// ------------------------------------------------------- persistent engine

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier of a cooperative launch (every block of the grid is
// resident).  One thread per block arrives; the last arrival resets the count
// and advances the generation.  Every wait is bounded: a wait that exceeds
// S->wait_limit_ns raises kSchedErrWait, and a wait ends early once any error
// bit is set.  Returns false in every thread of the block when an error bit is
// set.  `skip_arrive` (tests only) makes this block wait without arriving, so
// that every wait of this barrier runs out.
__device__ __forceinline__ bool grid_barrier(SchedState* S, bool skip_arrive, unsigned* flag_s) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &S->bar_gen;
        volatile unsigned* err = &S->error;
        const unsigned g = *gen;
        __threadfence();
        bool released = false;
        if (!skip_arrive) {
            const unsigned arrived = atomicAdd(&S->bar_count, 1u) + 1u;
            if (arrived == gridDim.x) {
                atomicExch(&S->bar_count, 0u);
                __threadfence();
                atomicAdd(&S->bar_gen, 1u);
                released = true;
            }
        }
        if (!released) {
            const unsigned long long t0 = global_ns();
            unsigned long long dt = 0;
            while (*gen == g && *err == 0) {
                dt = global_ns() - t0;
                if (dt > S->wait_limit_ns) {
                    atomicOr(&S->error, kSchedErrWait);
                    break;
                }
                __nanosleep(200);
            }
            if (dt > 0) atomicMax(&S->wait_seen_ns, dt);
        }
        __threadfence();
        *flag_s = *err;
    }
    __syncthreads();
    return *(volatile unsigned*)flag_s == 0;
}

// Chunks of depth d that no pass has consumed yet (deferred or fresh).
__device__ __forceinline__ unsigned long long sched_remaining(const SchedState* S, unsigned d) {
    const volatile SchedLevel* L = &S->lv[d];
    return (L->tail - L->head) + ((L->n_parents + 31) / 32 - L->fresh);
}

// The schedule step after a pass of depth d (one thread): account the pass's
// claims (consumed deferred entries leave the ring head, new deferrals were
// appended at its tail), then pick the next pass depth first -- descend into
// the level the pass just filled, else repeat d while it has chunks left,
// else return to the deepest ancestor with chunks left; 0 ends the match.
// `mid`: the pass wrote a next level.  `items`, `ring_count`, `def_room`: the
// pass's work items, deferred items among them and room for new deferrals.
__device__ __forceinline__ void sched_advance(SchedState* S, LaunchCtl* ctl_base, unsigned d, bool mid,
                                              unsigned long long items, unsigned long long ring_count,
                                              unsigned long long def_room, bool limit_hit) {
    volatile LaunchCtl* c = ctl_base + d;
    SchedLevel* L = &S->lv[d];
    const unsigned long long claimed = c->claim < items ? c->claim : items;
    const unsigned long long ring_claimed = claimed < ring_count ? claimed : ring_count;
    const unsigned long long ndef = c->ndef;
    L->head += ring_claimed;
    L->tail += ndef;
    L->fresh += claimed - ring_claimed;
    L->parents += c->parents;
    L->lookups += c->lookups;
    L->list_words += c->list_words;
    L->passes += 1;
    S->passes += 1;
    const unsigned long long produced = mid ? c->produced : 0;
    L->produced += produced;
    S->produced_total += produced;
    unsigned err = 0;
    if ((c->error & 1u) || ndef > def_room) err |= kSchedErrRing;
    if (c->error & 2u) err |= kSchedErrWait;      // a list stage's bounded wait ran out
    const unsigned long long left = sched_remaining(S, d);
    if (mid && produced == 0 && left == items && items > 0) err |= kSchedErrPool;
    if (limit_hit) err |= kSchedErrLimit;
    if (S->passes > kSchedMaxPasses) err |= kSchedErrPasses;
    // Past the work limit on partial matches, the rows already produced are
    // still carried down to the last level (whose own limit check stops the
    // count), but no level is resumed: the result is a lower bound.
    const bool over = S->work_limit && S->produced_total > S->work_limit;
    unsigned next = 0;
    if (!err) {
        if (mid && produced > 0) {
            next = d + 1;
            SchedLevel* N = &S->lv[next];
            N->n_parents = produced;
            N->fresh = 0;
            N->head = 0;
            N->tail = 0;
        } else if (over) {
            err |= kSchedErrLimit;
        } else {
            next = d;
            while (next >= 1 && sched_remaining(S, next) == 0) next--;
        }
    }
    if (next) {
        unsigned long long* w = (unsigned long long*)(ctl_base + next);
        for (unsigned i = 0; i < sizeof(LaunchCtl) / 8; i++) w[i] = 0;
    }
    if (err) atomicOr(&S->error, err);
    __threadfence();
    *(volatile unsigned*)&S->cur = next;
    __threadfence();
}

}  // namespace dev
}  // namespace fm
