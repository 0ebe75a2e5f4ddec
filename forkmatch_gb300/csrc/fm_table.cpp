// fm_table.cpp -- embedding-table files.
//
// The reference copies its table to the host and drops it (src/smsm.cu:1328-1348).
// Here a table can be written to a file for parity tooling: optionally sorted
// (lexicographic rows, so two runs or two systems compare byte for byte) and
// in either column layout -- the reference's (column i = vertex matched at the
// reference depth q-1-i, src/smsm.cu:743-760) or by query vertex id.
//
// File: "FMTB0001", u32 q, u32 columns (fm_columns), u64 rows, u32 sorted,
// u32 0, then rows x q u32, little-endian.
#include <algorithm>
#include <cstring>
#include <fstream>
#include <thread>
#include <vector>

#include "fm_internal.h"

using namespace fm;

namespace {

const char kTableMagic[8] = {'F', 'M', 'T', 'B', '0', '0', '0', '1'};
struct TableHeader {
    char magic[8];
    uint32_t q, columns;
    uint64_t rows;
    uint32_t sorted, reserved;
};
static_assert(sizeof(TableHeader) == 32, "table header layout");

// Row order by lexicographic compare, sorted in parallel chunks then merged.
std::vector<uint64_t> sorted_order(const uint32_t* rows, uint64_t n, uint32_t q) {
    std::vector<uint64_t> idx(n);
    for (uint64_t i = 0; i < n; i++) idx[i] = i;
    auto less = [rows, q](uint64_t a, uint64_t b) {
        const uint32_t* x = rows + a * q;
        const uint32_t* y = rows + b * q;
        for (uint32_t c = 0; c < q; c++)
            if (x[c] != y[c]) return x[c] < y[c];
        return false;
    };
    unsigned T = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < (1u << 16)) T = 1;
    std::vector<uint64_t> cut(T + 1);
    for (unsigned t = 0; t <= T; t++) cut[t] = n * t / T;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < T; t++)
        th.emplace_back([&, t] { std::sort(idx.begin() + cut[t], idx.begin() + cut[t + 1], less); });
    for (auto& x : th) x.join();
    for (unsigned width = 1; width < T; width *= 2) {
        std::vector<std::thread> mt;
        for (unsigned t = 0; t + width < T; t += 2 * width) {
            const uint64_t a = cut[t], m = cut[t + width], b = cut[std::min<unsigned>(t + 2 * width, T)];
            mt.emplace_back([&, a, m, b] { std::inplace_merge(idx.begin() + a, idx.begin() + m, idx.begin() + b, less); });
        }
        for (auto& x : mt) x.join();
    }
    return idx;
}

}  // namespace

extern "C" {

fm_status fm_table_write(const char* path, const uint32_t* rows, uint64_t n, uint32_t q, int32_t columns,
                         int32_t sort) {
    if (!path || (n && !rows) || q == 0 || q > FM_MAX_QUERY_VERTICES ||
        (columns != FM_COLUMNS_REFERENCE && columns != FM_COLUMNS_QUERY_ID))
        return FM_ERR_ARG;
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) {
        set_error(std::string("cannot write ") + path);
        return FM_ERR_IO;
    }
    TableHeader h;
    std::memcpy(h.magic, kTableMagic, 8);
    h.q = q;
    h.columns = (uint32_t)columns;
    h.rows = n;
    h.sorted = sort ? 1u : 0u;
    h.reserved = 0;
    f.write((const char*)&h, sizeof(h));
    if (!sort) {
        f.write((const char*)rows, (std::streamsize)(n * q * 4));
    } else {
        const std::vector<uint64_t> idx = sorted_order(rows, n, q);
        std::vector<uint32_t> buf;
        const uint64_t block = 1u << 16;
        for (uint64_t i = 0; i < n; i += block) {
            const uint64_t m = std::min(block, n - i);
            buf.resize(m * q);
            for (uint64_t r = 0; r < m; r++) std::memcpy(&buf[r * q], rows + idx[i + r] * q, q * 4);
            f.write((const char*)buf.data(), (std::streamsize)(m * q * 4));
        }
    }
    if (!f) {
        set_error(std::string("cannot write ") + path);
        return FM_ERR_IO;
    }
    return FM_OK;
}

fm_status fm_table_to_query_columns(const fm_query* query, const uint32_t* rows_ref, uint64_t n, uint32_t* rows_out) {
    if (!query || (n && (!rows_ref || !rows_out))) return FM_ERR_ARG;
    const Plan& p = query->p;
    const uint32_t q = p.q;
    // reference column i holds the image of the vertex matched at reference
    // depth q-1-i, i.e. of original vertex inv[order_local[q-1-i]]
    uint32_t dest[kMaxQ];
    for (uint32_t i = 0; i < q; i++) dest[i] = p.inv[p.order_local[q - 1 - i]];
    for (uint32_t i = 0; i < q; i++)
        if (dest[i] >= q) {
            set_error("query vertex ids are not 0..q-1");
            return FM_ERR_UNSUPPORTED;
        }
    std::vector<uint32_t> tmp(q);
    for (uint64_t r = 0; r < n; r++) {
        const uint32_t* src = rows_ref + r * q;
        for (uint32_t i = 0; i < q; i++) tmp[dest[i]] = src[i];
        std::memcpy(rows_out + r * q, tmp.data(), q * 4);
    }
    return FM_OK;
}

}  // extern "C"
