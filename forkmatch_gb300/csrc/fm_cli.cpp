// fm_cli.cpp -- `ForkMatch <query.g> <data.g>`, the reference's command line
// (src/smsm.cu:1351-1393 main, src/smsm.cu:1182-1349 match) on libforkmatch.
//
// Prints the reference's key stdout lines ("GPU Parse Time", "Parse Time",
// "Size of symmetry", "Kernel Time", "Soln Size", "End to End Time") and
// returns its exit codes: 99 wrong argument count, 12 missing data file,
// 76/77/78 data framing/header, 232/233/234 query file/format/missing lines,
// 1 disconnected or unsupported query or exhausted SOLN_PREALLOC.  Malformed
// data lines (where the reference traps on the device) return 79.
//
// Extras, all optional: FM_MODE=count (count only), FM_COLUMNS=query (table
// columns by query vertex id), FM_OUTPUT=<file> (write the table as an
// embedding-table file, fm_table_write; FM_OUTPUT_SORTED=1 sorts the rows),
// plus the FM_PREALLOC / FM_SOLN_PREALLOC / FM_OUTPUT_PREALLOC /
// FM_CUR_BANK_SIZE knobs.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "forkmatch.h"

static int exit_for_data(fm_status s) {
    switch (s) {
        case FM_ERR_IO: return 12;
        case FM_ERR_DATA_HEADER0: return 76;
        case FM_ERR_DATA_TRAILER: return 77;
        case FM_ERR_DATA_HEADER: return 78;
        case FM_ERR_DATA_LINE: return 79;
        default: return 1;
    }
}

static int exit_for_query(fm_status s) {
    switch (s) {
        case FM_ERR_IO: return 232;
        case FM_ERR_QUERY_FORMAT: return 233;
        case FM_ERR_QUERY_MISSING: return 234;
        default: return 1;
    }
}

static double secs(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
    return std::chrono::duration<double>(b - a).count();
}

int main(int argc, char** argv) {
    std::printf("Trie Graph Problem\n");
    if (argc != 3) return 99;
    auto t_start = std::chrono::steady_clock::now();
    const char* query_path = argv[1];
    const char* data_path = argv[2];
    std::printf("Query Graph - %s Data Graph - %s\n", query_path, data_path);

    fm_knobs knobs;
    fm_knobs_default(&knobs);
    fm_context* ctx = nullptr;
    fm_status st = fm_context_create(&knobs, &ctx);
    if (st != FM_OK) {
        std::printf("Error: %s (%s)\n", fm_status_string(st), fm_last_error());
        return 1;
    }
    auto t_parse = std::chrono::steady_clock::now();
    fm_graph* graph = nullptr;
    st = fm_graph_load_file(ctx, data_path, &graph);
    if (st != FM_OK) {
        if (st == FM_ERR_IO) std::printf("\nMissing file %s", data_path);
        else std::printf("Error: %s (%s)\n", fm_status_string(st), fm_last_error());
        fm_context_destroy(ctx);
        return exit_for_data(st);
    }
    fm_graph_info gi;
    fm_graph_get_info(graph, &gi);
    std::printf("GPU Parse Time: %f\n", gi.build_ms / 1000.0);

    fm_query* query = nullptr;
    st = fm_query_compile_file(query_path, &query);
    if (st != FM_OK) {
        if (st == FM_ERR_IO) std::printf("\nMissing file %s\n", query_path);
        else std::printf("Error: %s (%s)\n", fm_status_string(st), fm_last_error());
        fm_graph_free(graph);
        fm_context_destroy(ctx);
        return exit_for_query(st);
    }
    fm_query_info qi;
    fm_query_get_info(query, &qi);
    std::printf("\nSize of symmetry: %llu\n", (unsigned long long)qi.automorphisms);
    std::printf("\nMapping Order: ");
    for (uint32_t d = 0; d < qi.q; d++) std::printf("%u, ", qi.order[d]);
    std::printf("\n");
    auto t_parsed = std::chrono::steady_clock::now();
    std::printf("\nParse Time: %fs\n", secs(t_parse, t_parsed));

    fm_match_opts opts;
    fm_match_opts_default(&opts);
    const char* mode = std::getenv("FM_MODE");
    if (mode && std::strcmp(mode, "count") == 0) opts.mode = FM_MODE_COUNT;
    const char* cols = std::getenv("FM_COLUMNS");
    if (cols && std::strcmp(cols, "query") == 0) opts.columns = FM_COLUMNS_QUERY_ID;

    fm_result res;
    auto k0 = std::chrono::steady_clock::now();
    st = fm_match(ctx, graph, query, &opts, &res);
    auto k1 = std::chrono::steady_clock::now();
    if (st != FM_OK && st != FM_ERR_OUTPUT_OVERFLOW) {
        std::printf("Error: %s (%s)\n", fm_status_string(st), fm_last_error());
        fm_query_free(query);
        fm_graph_free(graph);
        fm_context_destroy(ctx);
        return 1;
    }
    std::printf("\nKernel Time: %fs\n", secs(k0, k1));
    std::printf("Soln Size: %llu\n", (unsigned long long)res.count);
    if (res.truncated)
        std::fprintf(stderr, "warning: table truncated to %llu rows (OUTPUT_PREALLOC)\n", (unsigned long long)res.rows);

    const char* outp = std::getenv("FM_OUTPUT");
    if (outp && *outp && opts.mode == FM_MODE_TABLE) {
        // copy through the library so no CUDA call is needed here, then write
        // an embedding-table file (FM_OUTPUT_SORTED=1: lexicographic rows)
        std::vector<uint32_t> rows(res.rows * res.q);
        fm_match_opts o2 = opts;
        o2.host_rows = rows.data();
        o2.host_rows_cap = res.rows;
        fm_result r2;
        fm_match(ctx, graph, query, &o2, &r2);
        const char* so = std::getenv("FM_OUTPUT_SORTED");
        const int sorted = so && std::strcmp(so, "1") == 0;
        if (fm_table_write(outp, rows.data(), r2.rows_copied, r2.q, opts.columns, sorted) != FM_OK)
            std::fprintf(stderr, "warning: %s\n", fm_last_error());
    }
    fm_query_free(query);
    fm_graph_free(graph);
    fm_context_destroy(ctx);
    std::printf("\nEnd to End Time: %fs\n", secs(t_start, std::chrono::steady_clock::now()));
    return 0;
}
