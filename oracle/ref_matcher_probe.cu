/*
 * ref_matcher_probe.cu -- TEST INFRASTRUCTURE: runs the reference's own GPU
 * matcher on one query and one data graph and prints what it found.
 *
 * The reference sources are compiled in place (never copied into this
 * repository) with SYMMETRY undefined: that build writes every embedding row
 * in the reference's column order and counts every embedding
 * (src/smsm.cu:706-779 isoWrite), while the default SYMMETRY build fills its
 * rows through a device buffer that is never initialised
 * (src/smsm.cu:1225-1227).  The reference copies its table to the host and
 * then drops it (src/smsm.cu:1338-1341); this probe records the last
 * device-to-host cudaMemcpy the reference makes (that table) and prints it.
 * The count and the "Kernel Time" are the reference's own stdout lines.
 *
 * Before matching, the probe clears the reference's preallocated slab: the
 * reference reads parts of it (trie bitmaps, the first offset) before writing
 * them and relies on fresh device memory being zero (src/trie.cuh:869).
 *
 * Output, after the reference's own lines: one line
 *   PROBE_ROWS <words> w0 w1 ...
 * with the u32 words of the table (rows of q words).
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

static void* g_last_d2h = nullptr;
static size_t g_last_d2h_bytes = 0;

static cudaError_t probe_memcpy(void* dst, const void* src, size_t n, cudaMemcpyKind kind) {
    cudaError_t e = cudaMemcpy(dst, src, n, kind);
    if (kind == cudaMemcpyDeviceToHost) {
        g_last_d2h = dst;
        g_last_d2h_bytes = n;
    }
    return e;
}

#include "environment.cuh"
#undef SYMMETRY
#define cudaMemcpy probe_memcpy
#define main reference_main
#include "smsm.cu"
#undef main
#undef cudaMemcpy

int main(int argc, char** argv) {
    if (argc != 3) return 99;
    if (cudaDeviceSetLimit(cudaLimitDevRuntimePendingLaunchCount, LaunchLimit) != cudaSuccess) return 98;
    unsigned char* slab = prealloc();
    if (cudaMemset(slab, 0, PREALLOC) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return 97;
    match(std::string(argv[1]), std::string(argv[2]), slab);
    if (cudaDeviceSynchronize() != cudaSuccess) return 96;
    const unsigned int* w = (const unsigned int*)g_last_d2h;
    const size_t words = g_last_d2h_bytes / sizeof(unsigned int);
    std::printf("\nPROBE_ROWS %zu", words);
    for (size_t i = 0; i < words; i++) std::printf(" %u", w[i]);
    std::printf("\n");
    std::fflush(stdout);
    return 0;
}
