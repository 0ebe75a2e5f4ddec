// fm_ingest.cu -- `.g` text parsed on the device.
//
// The reference parses its data file on the device too (parseCSR,
// src/trie.cuh:800-951), but with `int` offsets (src/trie.cuh:802,1115), so a
// file over 2 GiB cannot be read, and it never parses the first line after the
// header (src/trie.cuh:829-834,1176-1178).  Here every offset is 64-bit:
//
//   1. the host checks the framing ("t # 0\n", the header line, the trailing
//      "t # -1", the newline before it) -- a few bytes;
//   2. the body is copied to the device once;
//   3. k_count_lines / k_line_starts: each thread takes 16 bytes, a block scan
//      numbers the newlines, and every line start is written in file order;
//   4. k_parse_lines: one thread per line parses "v id label" or
//      "e src dst label" with the same grammar and range checks as the host
//      parser (fm_parse.cpp) and records the first bad line;
//   5. the kept e-lines (label < label slots) are compacted with CUB and go
//      straight to the device graph build, without a round trip to the host.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "fm_internal.h"

namespace fm {
namespace {

constexpr int kIngestBlock = 256;
constexpr uint64_t kBytesPerBlock = 16ull * kIngestBlock;   // 16 bytes per thread

__device__ __forceinline__ uint32_t newline_mask16(const unsigned char* b, uint64_t pos, uint64_t n, uint4& raw) {
    // 16 bytes starting at pos (pos is 16-aligned within the body buffer)
    uint32_t mask = 0;
    if (pos + 16 <= n) {
        raw = *reinterpret_cast<const uint4*>(b + pos);
        const uint32_t w[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (((w[i] >> (8 * j)) & 0xffu) == '\n') mask |= 1u << (4 * i + j);
    } else {
        for (uint64_t i = pos; i < n; i++)
            if (b[i] == '\n') mask |= 1u << (uint32_t)(i - pos);
    }
    return mask;
}

// Newlines per block of kBytesPerBlock bytes.
__global__ void k_count_lines(const unsigned char* __restrict__ body, uint64_t n, unsigned long long* __restrict__ per_block) {
    typedef cub::BlockReduce<uint32_t, kIngestBlock> Reduce;
    __shared__ typename Reduce::TempStorage tmp;
    const uint64_t pos = blockIdx.x * kBytesPerBlock + 16ull * threadIdx.x;
    uint4 raw;
    const uint32_t c = pos < n ? __popc(newline_mask16(body, pos, n, raw)) : 0u;
    const uint32_t s = Reduce(tmp).Sum(c);
    if (threadIdx.x == 0) per_block[blockIdx.x] = s;
}

// Start offset of every line: line 0 starts at 0, line i+1 after newline i.
__global__ void k_line_starts(const unsigned char* __restrict__ body, uint64_t n,
                              const unsigned long long* __restrict__ block_base, uint64_t* __restrict__ starts) {
    typedef cub::BlockScan<uint32_t, kIngestBlock> Scan;
    __shared__ typename Scan::TempStorage tmp;
    const uint64_t pos = blockIdx.x * kBytesPerBlock + 16ull * threadIdx.x;
    uint4 raw;
    uint32_t mask = pos < n ? newline_mask16(body, pos, n, raw) : 0u;
    uint32_t before = 0;
    Scan(tmp).ExclusiveSum(__popc(mask), before);
    uint64_t line = block_base[blockIdx.x] + before;   // newlines before this thread's bytes
    while (mask) {
        const int b = __ffs(mask) - 1;
        mask &= mask - 1;
        starts[line + 1] = pos + b + 1;
        line++;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) starts[0] = 0;
}

__device__ __forceinline__ bool dparse_u32(const unsigned char* b, uint64_t& p, uint64_t end, uint32_t& v) {
    uint64_t acc = 0;
    const uint64_t s = p;
    while (p < end && (unsigned char)(b[p] - '0') < 10) {
        acc = acc * 10 + (uint64_t)(b[p] - '0');
        if (acc > 0xffffffffull) return false;
        ++p;
    }
    if (p == s) return false;
    v = (uint32_t)acc;
    return true;
}

// One thread per line (lines [0, nlines), each ending with '\n').  An e-line
// that is kept writes its three values at its line index; flags[i] = 1 then.
__global__ void k_parse_lines(const unsigned char* __restrict__ body, const uint64_t* __restrict__ starts,
                              uint64_t nlines, uint32_t V, uint32_t EL, uint32_t L, uint32_t* __restrict__ src,
                              uint32_t* __restrict__ dst, uint32_t* __restrict__ lab, uint8_t* __restrict__ keep,
                              unsigned long long* __restrict__ first_bad) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nlines;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = starts[i];
        const uint64_t end = starts[i + 1];   // one past this line's '\n'
        bool ok = end >= p + 2;
        uint8_t k = 0;
        uint32_t v[3] = {0, 0, 0};
        if (ok) {
            const unsigned char kind = body[p];
            ok = (kind == 'v' || kind == 'e') && body[p + 1] == ' ';
            const int nv = kind == 'e' ? 3 : 2;
            p += 2;
            for (int f = 0; f < nv && ok; f++) {
                ok = dparse_u32(body, p, end, v[f]) && p < end && body[p] == ((f == nv - 1) ? '\n' : ' ');
                ++p;
            }
            if (ok) {
                if (kind == 'v') ok = v[0] < V;
                else ok = v[0] < V && v[1] < V && v[2] <= EL;
            }
            if (ok && kind == 'e' && v[2] < L) k = 1;
        }
        if (!ok) atomicMin(first_bad, (unsigned long long)i);
        keep[i] = k;
        src[i] = v[0];
        dst[i] = v[1];
        lab[i] = v[2];
    }
}

__global__ void k_label_hist(const uint32_t* __restrict__ lab, uint64_t n, unsigned long long* __restrict__ hist) {
    __shared__ unsigned int h[FM_MAX_LABEL + 1];
    for (uint32_t i = threadIdx.x; i <= FM_MAX_LABEL; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[lab[i] & FM_MAX_LABEL], 1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i <= FM_MAX_LABEL; i += blockDim.x)
        if (h[i]) atomicAdd(hist + i, (unsigned long long)h[i]);
}

struct DBuf {
    void* p = nullptr;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { reset(); }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
    }
    template <class T> T* as() { return (T*)p; }
};

fm_status dev_alloc(DBuf& b, uint64_t bytes) {
    if (cudaMalloc(&b.p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        set_error("cannot allocate device memory for parsing the data graph");
        return FM_ERR_NOMEM;
    }
    return FM_OK;
}

bool host_u32(const char*& p, const char* end, uint32_t& v) {
    uint64_t acc = 0;
    const char* s = p;
    while (p < end && (unsigned char)(*p - '0') < 10) {
        acc = acc * 10 + (uint64_t)(*p - '0');
        if (acc > 0xffffffffull) return false;
        ++p;
    }
    if (p == s) return false;
    v = (uint32_t)acc;
    return true;
}

}  // namespace

fm_status parse_data_text_device(const char* text, uint64_t len, cudaStream_t s, DeviceGraph& g) {
    // framing, checked on the host exactly as parse_data_text does
    if (len < 6 || std::memcmp(text, "t # 0\n", 6) != 0) {
        set_error("data graph does not start with \"t # 0\\n\"");
        return FM_ERR_DATA_HEADER0;
    }
    if (len < 12 || std::memcmp(text + len - 6, "t # -1", 6) != 0) {
        set_error("data graph does not end with \"t # -1\"");
        return FM_ERR_DATA_TRAILER;
    }
    const char* p = text + 6;
    const char* end = text + len - 6;
    uint32_t h[4] = {0, 0, 0, 0};
    for (int field = 0;; field++) {
        if (field > 3 || !host_u32(p, end, h[field]) || p >= end) {
            set_error("malformed data graph header");
            return FM_ERR_DATA_HEADER;
        }
        if (*p == '\n') {
            ++p;
            break;
        }
        if (*p != ' ') {
            set_error("malformed data graph header");
            return FM_ERR_DATA_HEADER;
        }
        ++p;
    }
    const uint32_t V = h[0];
    const uint64_t Ehdr = h[1];
    const uint32_t EL = h[3];
    const uint32_t L = std::min<uint32_t>(EL, FM_MAX_LABEL) + 1;
    const char* body = p;
    const uint64_t blen = (uint64_t)(end - body);
    if (blen && body[blen - 1] != '\n') {
        set_error("last data line is not terminated by a newline before \"t # -1\"");
        return FM_ERR_DATA_LINE;
    }

    int dev = 0, sms = 1;
    FM_CUDA(cudaGetDevice(&dev));
    FM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // body on the device (16-byte aligned, padded to whole 16-byte words)
    DBuf d_body;
    FM_TRY(dev_alloc(d_body, (blen + 31) & ~15ull));
    if (blen) FM_CUDA(cudaMemcpyAsync(d_body.p, body, blen, cudaMemcpyHostToDevice, s));
    const uint64_t nblocks = std::max<uint64_t>(1, (blen + kBytesPerBlock - 1) / kBytesPerBlock);
    if (nblocks > 0x7fffffffull) {
        set_error("data graph text too large");
        return FM_ERR_UNSUPPORTED;
    }
    DBuf d_cnt, d_base;
    FM_TRY(dev_alloc(d_cnt, nblocks * 8));
    FM_TRY(dev_alloc(d_base, nblocks * 8));
    const unsigned char* b = d_body.as<unsigned char>();
    k_count_lines<<<(unsigned)nblocks, kIngestBlock, 0, s>>>(b, blen, d_cnt.as<unsigned long long>());
    FM_CUDA(cudaGetLastError());
    size_t tb = 0;
    FM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, d_cnt.as<unsigned long long>(), d_base.as<unsigned long long>(),
                                          (int64_t)nblocks, s));
    DBuf d_tmp;
    FM_TRY(dev_alloc(d_tmp, tb));
    FM_CUDA(cub::DeviceScan::ExclusiveSum(d_tmp.p, tb, d_cnt.as<unsigned long long>(), d_base.as<unsigned long long>(),
                                          (int64_t)nblocks, s));
    unsigned long long last_base = 0, last_cnt = 0;
    FM_CUDA(cudaMemcpyAsync(&last_base, d_base.as<unsigned long long>() + (nblocks - 1), 8, cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaMemcpyAsync(&last_cnt, d_cnt.as<unsigned long long>() + (nblocks - 1), 8, cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaStreamSynchronize(s));
    const uint64_t nlines = last_base + last_cnt;   // every line ends with '\n'
    DBuf d_starts;
    FM_TRY(dev_alloc(d_starts, (nlines + 1) * 8));
    k_line_starts<<<(unsigned)nblocks, kIngestBlock, 0, s>>>(b, blen, d_base.as<unsigned long long>(),
                                                             d_starts.as<uint64_t>());
    FM_CUDA(cudaGetLastError());

    DBuf d_vals, d_keep, d_bad;
    FM_TRY(dev_alloc(d_vals, std::max<uint64_t>(1, nlines) * 12));
    FM_TRY(dev_alloc(d_keep, std::max<uint64_t>(1, nlines)));
    FM_TRY(dev_alloc(d_bad, 8));
    FM_CUDA(cudaMemsetAsync(d_bad.p, 0xff, 8, s));
    uint32_t* vsrc = d_vals.as<uint32_t>();
    uint32_t* vdst = vsrc + nlines;
    uint32_t* vlab = vdst + nlines;
    if (nlines) {
        const unsigned grid = (unsigned)std::min<uint64_t>((nlines + 255) / 256, (uint64_t)sms * 32);
        k_parse_lines<<<grid, 256, 0, s>>>(b, d_starts.as<uint64_t>(), nlines, V, EL, L, vsrc, vdst, vlab,
                                            d_keep.as<uint8_t>(), d_bad.as<unsigned long long>());
        FM_CUDA(cudaGetLastError());
    }
    unsigned long long bad = ~0ull;
    FM_CUDA(cudaMemcpyAsync(&bad, d_bad.p, 8, cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaStreamSynchronize(s));
    if (bad != ~0ull) {
        uint64_t at = 0;
        FM_CUDA(cudaMemcpy(&at, d_starts.as<uint64_t>() + bad, 8, cudaMemcpyDeviceToHost));
        const char* line = body + at;
        const char* nl = (const char*)std::memchr(line, '\n', (size_t)(end - line));
        std::string txt(line, nl ? (size_t)(nl - line) : std::min<size_t>(40, (size_t)(end - line)));
        set_error("malformed or out-of-range data line: \"" + txt.substr(0, 80) + "\"");
        return FM_ERR_DATA_LINE;
    }
    d_starts.reset();
    d_body.reset();

    // compact the kept e-lines (three flagged selections share the flags)
    DBuf d_edges, d_nsel;
    FM_TRY(dev_alloc(d_edges, std::max<uint64_t>(1, nlines) * 12));
    FM_TRY(dev_alloc(d_nsel, 8));
    uint32_t* esrc = d_edges.as<uint32_t>();
    uint32_t* edst = esrc + nlines;
    uint32_t* elab = edst + nlines;
    uint64_t E = 0;
    if (nlines) {
        size_t tb2 = 0;
        FM_CUDA(cub::DeviceSelect::Flagged(nullptr, tb2, vsrc, d_keep.as<uint8_t>(), esrc,
                                           d_nsel.as<unsigned long long>(), (int64_t)nlines, s));
        DBuf d_tmp2;
        FM_TRY(dev_alloc(d_tmp2, tb2));
        FM_CUDA(cub::DeviceSelect::Flagged(d_tmp2.p, tb2, vsrc, d_keep.as<uint8_t>(), esrc,
                                           d_nsel.as<unsigned long long>(), (int64_t)nlines, s));
        FM_CUDA(cub::DeviceSelect::Flagged(d_tmp2.p, tb2, vdst, d_keep.as<uint8_t>(), edst,
                                           d_nsel.as<unsigned long long>(), (int64_t)nlines, s));
        FM_CUDA(cub::DeviceSelect::Flagged(d_tmp2.p, tb2, vlab, d_keep.as<uint8_t>(), elab,
                                           d_nsel.as<unsigned long long>(), (int64_t)nlines, s));
        unsigned long long ne = 0;
        FM_CUDA(cudaMemcpyAsync(&ne, d_nsel.p, 8, cudaMemcpyDeviceToHost, s));
        FM_CUDA(cudaStreamSynchronize(s));
        E = ne;
    }
    if (E > Ehdr) {
        set_error("more e-lines than the header's edge count");
        return FM_ERR_DATA_LINE;
    }
    d_vals.reset();
    d_keep.reset();
    // label frequencies for the matching-order cost model
    DBuf d_hist;
    FM_TRY(dev_alloc(d_hist, (FM_MAX_LABEL + 1) * 8));
    FM_CUDA(cudaMemsetAsync(d_hist.p, 0, (FM_MAX_LABEL + 1) * 8, s));
    if (E) {
        k_label_hist<<<(unsigned)std::min<uint64_t>((E + 255) / 256, (uint64_t)sms * 8), 256, 0, s>>>(
            elab, E, d_hist.as<unsigned long long>());
        FM_CUDA(cudaGetLastError());
    }
    std::vector<unsigned long long> hist(FM_MAX_LABEL + 1);
    FM_CUDA(cudaMemcpyAsync(hist.data(), d_hist.p, hist.size() * 8, cudaMemcpyDeviceToHost, s));
    FM_CUDA(cudaStreamSynchronize(s));
    fm_status st = build_device_graph(g, V, L, E, esrc, edst, elab, s);
    cudaStreamSynchronize(s);
    if (st != FM_OK) return st;
    g.label_count.assign(L, 0);
    for (uint32_t l = 0; l < L; l++) g.label_count[l] = hist[l];
    return FM_OK;
}

}  // namespace fm
