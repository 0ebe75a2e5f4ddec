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
        const uint32_t c = (s.x > 0 && s.y == x) + (s.x > 1 && s.z == x) + (s.x > 2 && s.w == x);
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

}  // namespace dev
}  // namespace fm
