// fm_graph.cu -- device build of the resident data graph.
//
// The reference builds one global CSR over (label, src) sorted by
// (label, src, dst), indexed through a per-label 32-vertex presence bitmap plus
// popcount rank (src/trie.cuh:138-311, 697-795, 898-942): a lookup costs two
// dependent loads before the list itself.  Here every (label, vertex) pair has a
// 16-byte segment record in a dense [label][vertex] table, so a lookup is one
// vectorised load; lists of up to 3 neighbours live inside the record (no
// second access), longer lists start on a 16-byte boundary in `nbr`.
// Sorting uses CUB's radix sort (graph build is not on the matching path).
#include <cstdlib>

#include <cub/cub.cuh>

#include "fm_internal.h"

namespace fm {
namespace {

__global__ void k_make_keys(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst,
                            const uint32_t* __restrict__ lab, uint64_t E, uint32_t V, uint32_t L,
                            uint32_t vbits, uint64_t* __restrict__ keys, unsigned int* err, unsigned int* loops) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = src[i], d = dst[i], l = lab[i];
        if (s >= V || d >= V || l >= L) {
            atomicOr(err, 1u);
            s = d = l = 0;
        } else if (s == d) {
            atomicOr(loops, 1u);
        }
        keys[i] = ((uint64_t)l << (2 * vbits)) | ((uint64_t)s << vbits) | (uint64_t)d;
    }
}

__global__ void k_heads(const uint64_t* __restrict__ keys, uint64_t E, uint32_t vbits, uint32_t* __restrict__ head,
                        unsigned int* dup) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k = keys[i];
        uint32_t h = 1;
        if (i > 0) {
            uint64_t p = keys[i - 1];
            h = (k >> vbits) != (p >> vbits);
            if (k == p) *dup = 1u;
        }
        head[i] = h;
    }
}

__global__ void k_seg_starts(const uint32_t* __restrict__ head, const uint32_t* __restrict__ incl, uint64_t E,
                             uint64_t* __restrict__ seg_start) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        if (head[i]) seg_start[incl[i] - 1] = i;
    }
}

__global__ void k_seg_len16(const uint64_t* __restrict__ seg_start, uint64_t nseg, uint64_t E,
                            uint64_t* __restrict__ len16, unsigned int* max_len, unsigned long long* nlong) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nseg; s += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t b = seg_start[s];
        uint64_t e = (s + 1 < nseg) ? seg_start[s + 1] : E;
        uint64_t n = e - b;
        len16[s] = n > 3 ? (n + 3) / 4 : 0;
        atomicMax(max_len, (unsigned int)n);
        if (n > 3) atomicAdd(nlong, 1ull);
    }
}

__global__ void k_fill_segments(const uint64_t* __restrict__ keys, const uint64_t* __restrict__ seg_start,
                                const uint64_t* __restrict__ off16, uint64_t nseg, uint64_t E, uint32_t V,
                                uint32_t vbits, uint4* __restrict__ seg) {
    const uint64_t vmask = (1ull << vbits) - 1;
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nseg; s += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t b = seg_start[s];
        uint64_t e = (s + 1 < nseg) ? seg_start[s + 1] : E;
        uint32_t n = (uint32_t)(e - b);
        uint64_t k = keys[b];
        uint32_t src = (uint32_t)((k >> vbits) & vmask);
        uint32_t lab = (uint32_t)(k >> (2 * vbits));
        uint4 r;
        r.x = n;
        if (n <= 3) {
            r.y = (uint32_t)(keys[b] & vmask);
            r.z = n > 1 ? (uint32_t)(keys[b + 1] & vmask) : kNoVertex;
            r.w = n > 2 ? (uint32_t)(keys[b + 2] & vmask) : kNoVertex;
        } else {
            r.y = (uint32_t)off16[s];
            r.z = (uint32_t)(keys[b] & vmask);
            r.w = (uint32_t)(keys[e - 1] & vmask);
        }
        seg[(uint64_t)lab * V + src] = r;
    }
}

__global__ void k_copy_long(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ incl,
                            const uint64_t* __restrict__ seg_start, const uint64_t* __restrict__ off16, uint64_t nseg,
                            uint64_t E, uint32_t vbits, uint32_t* __restrict__ nbr) {
    const uint64_t vmask = (1ull << vbits) - 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t s = incl[i] - 1;
        uint64_t b = seg_start[s];
        uint64_t e = (s + 1 < nseg) ? seg_start[s + 1] : E;
        uint64_t n = e - b;
        if (n <= 3) continue;
        uint32_t* dst = nbr + off16[s] * 4;
        dst[i - b] = (uint32_t)(keys[i] & vmask);
        if (i == b) {
            for (uint64_t j = n; j < ((n + 3) & ~3ull); j++) dst[j] = kNoVertex;
        }
    }
}

// Source vertex of each segment (segments are in (label, src) order) and the
// first segment of every label that has one (one writer per label).
__global__ void k_seg_heads(const uint64_t* __restrict__ keys, const uint64_t* __restrict__ seg_start, uint64_t nseg,
                            uint32_t vbits, uint32_t* __restrict__ heads, unsigned long long* __restrict__ first) {
    const uint64_t vmask = (1ull << vbits) - 1;
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nseg; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[seg_start[s]];
        heads[s] = (uint32_t)((k >> vbits) & vmask);
        const uint32_t l = (uint32_t)(k >> (2 * vbits));
        if (s == 0 || (uint32_t)(keys[seg_start[s - 1]] >> (2 * vbits)) != l) first[l] = s;
    }
}

// Lists of at least 2^min_log2 entries, counted by floor(log2(length)).
__global__ void k_len_hist(const uint64_t* __restrict__ seg_start, uint64_t nseg, uint64_t E, uint32_t min_log2,
                           unsigned int* __restrict__ hist) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nseg; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t n = ((s + 1 < nseg) ? seg_start[s + 1] : E) - seg_start[s];
        if (n >> min_log2) atomicAdd(hist + (63 - __clzll((long long)n)), 1u);
    }
}

// Give every list of at least `thresh` entries a bitmap index (marked in the
// z field of its record) and remember where its entries live.
__global__ void k_bm_assign(const uint64_t* __restrict__ keys, const uint64_t* __restrict__ seg_start,
                            const uint64_t* __restrict__ off16, uint64_t nseg, uint64_t E, uint32_t V, uint32_t vbits,
                            uint64_t thresh, uint32_t cap, unsigned int* __restrict__ counter, uint4* __restrict__ seg,
                            uint2* __restrict__ bm_list) {
    const uint64_t vmask = (1ull << vbits) - 1;
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nseg; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = seg_start[s];
        const uint64_t n = ((s + 1 < nseg) ? seg_start[s + 1] : E) - b;
        if (n < thresh || n <= 3) continue;
        const unsigned int idx = atomicAdd(counter, 1u);
        if (idx >= cap) continue;
        const uint64_t k = keys[b];
        const uint32_t src = (uint32_t)((k >> vbits) & vmask);
        const uint32_t lab = (uint32_t)(k >> (2 * vbits));
        reinterpret_cast<uint32_t*>(seg + (uint64_t)lab * V + src)[2] = kBitmapMark | idx;
        bm_list[idx] = make_uint2((uint32_t)off16[s], (uint32_t)n);
    }
}

// One block per bitmap: set the bit of every entry.
__global__ void k_bm_fill(const uint32_t* __restrict__ nbr, const uint2* __restrict__ bm_list, uint32_t n_bm,
                          uint32_t bm_words, uint32_t* __restrict__ bitmaps) {
    for (uint32_t i = blockIdx.x; i < n_bm; i += gridDim.x) {
        const uint2 e = bm_list[i];
        const uint32_t* list = nbr + (uint64_t)e.x * 4;
        uint32_t* bits = bitmaps + (uint64_t)i * bm_words;
        for (uint32_t t = threadIdx.x; t < e.y; t += blockDim.x) {
            const uint32_t x = list[t];
            atomicOr(bits + (x >> 5), 1u << (x & 31));
        }
    }
}

uint32_t bits_for(uint64_t x) {   // bits needed to store values 0..x
    uint32_t b = 1;
    while (b < 64 && (x >> b)) ++b;
    return b;
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    template <class T> T* as() { return (T*)p; }
};

uint64_t env_bytes(const char* name, uint64_t dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    char* end = nullptr;
    const unsigned long long x = std::strtoull(v, &end, 10);
    return (end && *end == 0) ? (uint64_t)x : dflt;
}

// Out-of-line (long) list count so far (device counter), read back.
uint64_t nlong_hint(const unsigned long long* d_nlong, cudaStream_t s) {
    unsigned long long n = 0;
    if (cudaMemcpyAsync(&n, d_nlong, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return 1;
    return n;
}

int grid_for(uint64_t n, int sms) {
    uint64_t b = (n + 255) / 256;
    uint64_t cap = (uint64_t)sms * 32;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace

fm_status build_device_graph(DeviceGraph& g, uint32_t V, uint32_t L, uint64_t E, const uint32_t* d_src,
                             const uint32_t* d_dst, const uint32_t* d_lab, cudaStream_t s) {
    if (V == 0 || L == 0) {
        set_error("graph needs at least one vertex and one label slot");
        return FM_ERR_ARG;
    }
    const uint32_t vbits = bits_for(V - 1);
    const uint32_t lbits = bits_for(L - 1);
    if (2 * vbits + lbits > 64) {
        set_error("vertex and label ids do not fit the 64-bit sort key");
        return FM_ERR_UNSUPPORTED;
    }
    if (E >= (1ull << 32)) {
        set_error("more than 2^32 - 1 directed e-lines");
        return FM_ERR_UNSUPPORTED;
    }
    int dev = 0, sms = 1;
    FM_CUDA(cudaGetDevice(&dev));
    FM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaEvent_t ev0, ev1;
    FM_CUDA(cudaEventCreate(&ev0));
    FM_CUDA(cudaEventCreate(&ev1));
    FM_CUDA(cudaEventRecord(ev0, s));

    g = DeviceGraph();
    g.V = V;
    g.L = L;
    g.E = E;
    g.vbits = vbits;
    g.device = dev;
    FM_CUDA(cudaMalloc(&g.seg, (size_t)L * V * sizeof(uint4)));
    FM_CUDA(cudaMemsetAsync(g.seg, 0, (size_t)L * V * sizeof(uint4), s));

    DevBuf flags;   // [0] error, [1] dup, [2] max_len, [3] self-loop seen, [4..5] nlong
    FM_CUDA(cudaMalloc(&flags.p, 64));
    FM_CUDA(cudaMemsetAsync(flags.p, 0, 64, s));
    unsigned int* d_err = flags.as<unsigned int>();
    unsigned int* d_dup = d_err + 1;
    unsigned int* d_max = d_err + 2;
    unsigned int* d_loops = d_err + 3;
    unsigned long long* d_nlong = (unsigned long long*)(d_err + 4);

    uint64_t nseg = 0, total16 = 0;
    if (E > 0) {
        DevBuf keys, keys_alt, temp, head, incl;
        FM_CUDA(cudaMalloc(&keys.p, E * 8));
        FM_CUDA(cudaMalloc(&keys_alt.p, E * 8));
        k_make_keys<<<grid_for(E, sms), 256, 0, s>>>(d_src, d_dst, d_lab, E, V, L, vbits, keys.as<uint64_t>(), d_err,
                                                     d_loops);
        FM_CUDA(cudaGetLastError());
        cub::DoubleBuffer<uint64_t> db(keys.as<uint64_t>(), keys_alt.as<uint64_t>());
        size_t tb = 0;
        FM_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb, db, (int64_t)E, 0, (int)(2 * vbits + lbits), s));
        FM_CUDA(cudaMalloc(&temp.p, tb));
        FM_CUDA(cub::DeviceRadixSort::SortKeys(temp.p, tb, db, (int64_t)E, 0, (int)(2 * vbits + lbits), s));
        const uint64_t* sorted = db.Current();
        FM_CUDA(cudaMalloc(&head.p, E * 4));
        FM_CUDA(cudaMalloc(&incl.p, E * 4));
        k_heads<<<grid_for(E, sms), 256, 0, s>>>(sorted, E, vbits, head.as<uint32_t>(), d_dup);
        FM_CUDA(cudaGetLastError());
        size_t tb2 = 0;
        FM_CUDA(cub::DeviceScan::InclusiveSum(nullptr, tb2, head.as<uint32_t>(), incl.as<uint32_t>(), (int64_t)E, s));
        DevBuf temp2;
        FM_CUDA(cudaMalloc(&temp2.p, tb2));
        FM_CUDA(cub::DeviceScan::InclusiveSum(temp2.p, tb2, head.as<uint32_t>(), incl.as<uint32_t>(), (int64_t)E, s));
        uint32_t nseg32 = 0, dup_seen = 0;
        FM_CUDA(cudaMemcpyAsync(&nseg32, incl.as<uint32_t>() + (E - 1), 4, cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaMemcpyAsync(&dup_seen, d_dup, 4, cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        nseg = nseg32;
        DevBuf seg_start, len16, off16;
        FM_CUDA(cudaMalloc(&seg_start.p, nseg * 8));
        FM_CUDA(cudaMalloc(&len16.p, nseg * 8));
        FM_CUDA(cudaMalloc(&off16.p, nseg * 8));
        k_seg_starts<<<grid_for(E, sms), 256, 0, s>>>(head.as<uint32_t>(), incl.as<uint32_t>(), E,
                                                     seg_start.as<uint64_t>());
        k_seg_len16<<<grid_for(nseg, sms), 256, 0, s>>>(seg_start.as<uint64_t>(), nseg, E, len16.as<uint64_t>(),
                                                       d_max, d_nlong);
        FM_CUDA(cudaGetLastError());
        size_t tb3 = 0;
        FM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb3, len16.as<uint64_t>(), off16.as<uint64_t>(), (int64_t)nseg, s));
        DevBuf temp3;
        FM_CUDA(cudaMalloc(&temp3.p, tb3));
        FM_CUDA(cub::DeviceScan::ExclusiveSum(temp3.p, tb3, len16.as<uint64_t>(), off16.as<uint64_t>(), (int64_t)nseg, s));
        uint64_t last_off = 0, last_len = 0;
        FM_CUDA(cudaMemcpyAsync(&last_off, off16.as<uint64_t>() + (nseg - 1), 8, cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaMemcpyAsync(&last_len, len16.as<uint64_t>() + (nseg - 1), 8, cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        total16 = last_off + last_len;
        if (total16 >= (1ull << 32)) {
            set_error("out-of-line neighbour storage exceeds 64 GiB");
            return FM_ERR_UNSUPPORTED;
        }
        g.nbr_words = total16 * 4;
        FM_CUDA(cudaMalloc(&g.nbr, (g.nbr_words ? g.nbr_words : 4) * 4));
        k_fill_segments<<<grid_for(nseg, sms), 256, 0, s>>>(sorted, seg_start.as<uint64_t>(), off16.as<uint64_t>(),
                                                           nseg, E, V, vbits, g.seg);
        k_copy_long<<<grid_for(E, sms), 256, 0, s>>>(sorted, incl.as<uint32_t>(), seg_start.as<uint64_t>(),
                                                    off16.as<uint64_t>(), nseg, E, vbits, g.nbr);
        FM_CUDA(cudaGetLastError());
        DevBuf per_label;
        FM_CUDA(cudaMalloc(&g.heads, nseg * 4));
        FM_CUDA(cudaMalloc(&per_label.p, (size_t)L * 8));
        FM_CUDA(cudaMemsetAsync(per_label.p, 0xff, (size_t)L * 8, s));
        k_seg_heads<<<grid_for(nseg, sms), 256, 0, s>>>(sorted, seg_start.as<uint64_t>(), nseg, vbits, g.heads,
                                                       per_label.as<unsigned long long>());
        FM_CUDA(cudaGetLastError());
        std::vector<unsigned long long> first(L);
        FM_CUDA(cudaMemcpyAsync(first.data(), per_label.p, (size_t)L * 8, cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        // a label without segments starts where the next label with one does
        g.head_off.assign(L + 1, nseg);
        for (uint32_t l = L; l-- > 0;) g.head_off[l] = first[l] != ~0ull ? first[l] : g.head_off[l + 1];

        // membership bitmaps for the longest lists (not with duplicates: a
        // bit cannot count copies; vertex ids must leave bit 31 of z free)
        // default budget: room for 16384 bitmaps, between 2 and 8 GiB (on a
        // 2^22-vertex R-MAT graph with 64 labels, 8 GiB covers its 16256
        // lists of 256+ entries and measured faster than 2 GiB for every
        // query class, while 61 GB of bitmaps down to 64 entries slowed the
        // table queries)
        const uint32_t words = (V + 31) / 32;
        const uint64_t budget = env_bytes(
            "FM_BITMAP_BYTES", std::min<uint64_t>(8ull << 30, std::max<uint64_t>(2ull << 30, 16384ull * 4ull * words)));
        const uint64_t min_len = std::max<uint64_t>(4, env_bytes("FM_BITMAP_MIN_LEN", 64));
        const uint64_t cap64 = budget / (4ull * words);
        if (!dup_seen && V < kBitmapMark && cap64 > 0 && nlong_hint(d_nlong, s) > 0) {
            uint32_t min_log2 = 0;
            while ((1ull << min_log2) < min_len) min_log2++;
            DevBuf hist;
            FM_CUDA(cudaMalloc(&hist.p, 64 * 4 + 4));
            FM_CUDA(cudaMemsetAsync(hist.p, 0, 64 * 4 + 4, s));
            k_len_hist<<<grid_for(nseg, sms), 256, 0, s>>>(seg_start.as<uint64_t>(), nseg, E, min_log2,
                                                          hist.as<unsigned int>());
            FM_CUDA(cudaGetLastError());
            unsigned int h[64];
            FM_CUDA(cudaMemcpyAsync(h, hist.p, sizeof(h), cudaMemcpyDeviceToHost, s));
            FM_CUDA(cudaStreamSynchronize(s));
            const uint32_t cap = (uint32_t)std::min<uint64_t>(cap64, 1u << 30);
            // smallest power-of-two threshold whose lists all fit the budget
            uint64_t above = 0;
            int pick = -1;
            for (int b = 63; b >= (int)min_log2; b--) {
                if (above + h[b] > cap) break;
                above += h[b];
                if (h[b]) pick = b;
            }
            if (pick >= 0 && above > 0) {
                const uint64_t thresh = 1ull << pick;
                uint64_t n_bm = 0;
                for (int b = pick; b < 64; b++) n_bm += h[b];
                DevBuf bm_list;
                FM_CUDA(cudaMalloc(&bm_list.p, n_bm * sizeof(uint2)));
                FM_CUDA(cudaMalloc(&g.bitmaps, n_bm * words * 4ull));
                FM_CUDA(cudaMemsetAsync(g.bitmaps, 0, n_bm * words * 4ull, s));
                unsigned int* counter = hist.as<unsigned int>() + 64;
                k_bm_assign<<<grid_for(nseg, sms), 256, 0, s>>>(sorted, seg_start.as<uint64_t>(), off16.as<uint64_t>(),
                                                               nseg, E, V, vbits, thresh, (uint32_t)n_bm, counter,
                                                               g.seg, bm_list.as<uint2>());
                FM_CUDA(cudaGetLastError());
                const uint32_t fill_grid = (uint32_t)std::min<uint64_t>(n_bm, (uint64_t)sms * 16);
                k_bm_fill<<<fill_grid, 256, 0, s>>>(g.nbr, bm_list.as<uint2>(), (uint32_t)n_bm, words, g.bitmaps);
                FM_CUDA(cudaGetLastError());
                FM_CUDA(cudaStreamSynchronize(s));
                g.n_bitmaps = (uint32_t)n_bm;
                g.bm_words = words;
                g.bm_min_len = (uint32_t)thresh;
            }
        }
    } else {
        FM_CUDA(cudaMalloc(&g.nbr, 16));
        FM_CUDA(cudaMalloc(&g.heads, 16));
        g.head_off.assign(L + 1, 0);
    }
    unsigned int hflags[4] = {0, 0, 0, 0};
    unsigned long long nlong = 0;
    FM_CUDA(cudaMemcpyAsync(hflags, d_err, 16, cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaMemcpyAsync(&nlong, d_nlong, 8, cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaEventRecord(ev1, s));
    FM_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (hflags[0]) {
        set_error("edge endpoint or label out of range");
        return FM_ERR_DATA_LINE;
    }
    g.has_dups = hflags[1] ? 1 : 0;
    g.has_self_loops = hflags[3] ? 1 : 0;
    g.max_len = hflags[2];
    g.segments = nseg;
    g.long_segments = nlong;
    g.build_ms = ms;
    return FM_OK;
}

}  // namespace fm
