/*
 * ref_planner_probe.cu -- TEST INFRASTRUCTURE: drives the reference's own host
 * query planner, compiled from the ForkMatch sources in place (never copied),
 * and prints what it computed as one JSON line.  Used only to pin the oracle's
 * planner restatement (src/hostparser.cuh:286-508 fileParse,
 * src/ccsr.cuh:485-728 preProcessQuery).  The process exit code is the
 * reference's own when its planner calls exit().
 */
#include <cstdio>
#include <cstring>
#include <set>
#include <random>
#include "environment.cuh"
#undef info_printf
#define info_printf(f_, ...) do {} while (0)
#include "hostparser.cuh"

int main(int argc, char** argv) {
    if (argc != 2) return 99;
    CCSR query;
    fileParse(argv[1], &query, false);
    Requirements req;
    unsigned maxValency = preProcessQuery(query, &req);
    unsigned q = query.count;
    std::printf("{\"rc\": 0, \"q\": %u, \"max_valency\": %u, \"sym_count\": %u, \"aut_count\": %zu, \"inv\": [",
                q, maxValency, req.symmetryCount, symmetries.size());
    for (unsigned i = 0; i < q; i++) std::printf("%s%u", i ? ", " : "", query.invVertices[i]);
    std::printf("], \"mapping\": [");
    for (unsigned i = 0; i < q; i++) std::printf("%s%d", i ? ", " : "", req.mappingData[i]);
    std::printf("], \"headers\": [");
    for (unsigned i = 0; i < q; i++)
        std::printf("%s[%u, %u, %u, %u]", i ? ", " : "", req.header[i].count, req.header[i].index,
                    req.header[i].pkDist, req.header[i].lastSymmetry);
    std::printf("], \"reqs\": [");
    for (unsigned i = 0; i < req.size / 3; i++)
        std::printf("%s[%u, %u, %u]", i ? ", " : "", req.reqs[3 * i], req.reqs[3 * i + 1], req.reqs[3 * i + 2]);
    std::printf("]}\n");
    return 0;
}
