/*
 * fm_oracle.h -- CPU oracle for the ForkMatch hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * algorithm, used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline as the checker.  The product library (libforkmatch) never links,
 * loads or calls anything here.
 *
 * What it restates (paths relative to the ForkMatch source tree):
 *   - data-graph .g parsing: src/trie.cuh:999-1023 (parseHeader),
 *     src/trie.cuh:1051-1222 (parseGraph), src/trie.cuh:800-951 (parseCSR line
 *     grammar, parseNum src/trie.cuh:652-664);
 *   - the per-(label, source) sorted neighbour lists of the trie CSR:
 *     src/trie.cuh:266-310 (neighbours), src/trie.cuh:750-795 (csrToTrie),
 *     ordering key (label, src, dst) src/trie.cuh:89-115;
 *   - query .g parsing and vertex ordering: src/hostparser.cuh:190-266
 *     (parseValues), src/hostparser.cuh:286-508 (fileParse), src/hostparser.cuh:20-30
 *     (OrderPair: degree desc, then id asc);
 *   - the matching order and per-depth requirements:
 *     src/ccsr.cuh:229-326 (genereateCCSRRequirements), src/ccsr.cuh:485-549,
 *     src/ccsr.cuh:681-693 (climb delta encoding), src/ccsr.cuh:719-725 (validation);
 *   - automorphisms and the reference's symmetry breaking:
 *     src/ccsr.cuh:383-465 (queryMatch), src/ccsr.cuh:553-673 (identity,
 *     equivalent groups, lastSymmetry), src/smsm.cu:188-227 (isInj);
 *   - the matcher: roots src/smsm.cu:786-867 (isoInit), list intersection
 *     src/smsm.cu:57-140,299-345 (hasNext/isoCompare/isoGen: a k-way merge, so
 *     a value present in every list is produced min(multiplicity) times),
 *     injectivity src/smsm.cu:188-227, count and table src/smsm.cu:706-779
 *     (isoWrite: column i holds the image of the vertex matched at depth q-1-i).
 *
 * Parity pinning: the planner restatement is checked against the reference's
 * own host planner compiled from its sources (oracle/_ref/ref_planner, built by
 * oracle/build.py) on the reference's query fixtures; the matcher is checked
 * against closed-form counts (complete graphs, stars, cycles).  The reference
 * ships no golden match outputs, so match counts are pinned by those
 * known-answer tests rather than by reference output.
 */
#ifndef FM_ORACLE_H
#define FM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAXQ 32

typedef struct ora_graph ora_graph;

/* Reference exit codes reproduced by the parsers (src/trie.cuh:1059-1092,
 * src/hostparser.cuh:15-18,292-387, src/ccsr.cuh:252-254,581-583,719-725). */
enum {
    ORA_OK = 0,
    ORA_EXIT_PLAN = 1,        /* disconnected query / planner failure */
    ORA_EXIT_DATA_MISSING = 12,
    ORA_EXIT_DATA_HEADER0 = 76,
    ORA_EXIT_DATA_TRAILER = 77,
    ORA_EXIT_DATA_HEADER = 78,
    ORA_EXIT_DATA_LINE = 79,  /* reference traps (SAFEPARSE); oracle reports it */
    ORA_EXIT_QUERY_MISSING = 232,
    ORA_EXIT_QUERY_INVALID = 233,
    ORA_EXIT_QUERY_MISSING_DATA = 234,
    ORA_EXIT_NO_IDENTITY = 999,
    ORA_EXIT_LIMIT = 1000     /* ora_match stopped at one of its search limits */
};

/* Build from directed e-lines (both directions must be listed by the caller,
 * as the .g format requires).  Duplicates are kept. */
int ora_graph_from_edges(uint32_t V, uint32_t n_labels, uint64_t E,
                         const uint32_t* src, const uint32_t* dst,
                         const uint32_t* label, ora_graph** out);
/* Parse .g text (whole file contents). */
int ora_graph_parse(const char* text, size_t len, ora_graph** out);
void ora_graph_free(ora_graph* g);
uint32_t ora_graph_vertices(const ora_graph* g);
uint64_t ora_graph_edges(const ora_graph* g);
uint32_t ora_graph_labels(const ora_graph* g);
/* Neighbour list of (label, v): returns its length and sets *ptr. */
uint64_t ora_graph_list(const ora_graph* g, uint32_t label, uint32_t v, const uint32_t** ptr);
/* Vertices with a non-empty list of `label`. */
uint32_t ora_graph_sources(const ora_graph* g, uint32_t label);

typedef struct {
    int q;                          /* query vertices */
    int max_valency;                /* longest CCSR row (out-degree) */
    int inv[ORA_MAXQ];              /* local index -> original query vertex id */
    int order[ORA_MAXQ];            /* local vertex matched at depth d */
    int ref_mapping[ORA_MAXQ];      /* reference mappingData: local vertex matched at depth q-1-i */
    int nreq[ORA_MAXQ];             /* requirements (back edges) per depth */
    int req_climb[ORA_MAXQ][ORA_MAXQ];   /* absolute climb (depth distance) */
    int req_label[ORA_MAXQ][ORA_MAXQ];   /* label of new->ancestor e-line: the list N_label(f(anc)) */
    int req_refl[ORA_MAXQ][ORA_MAXQ];    /* label of ancestor->new e-line */
    int pk_dist[ORA_MAXQ];          /* reference header pkDist */
    int last_sym[ORA_MAXQ];         /* reference lastSymmetry per depth (0 = none) */
    uint64_t aut_count;             /* |Aut| by the reference's enumeration (0 if not enumerated) */
    uint64_t sym_count;             /* reference symmetryCount (1 when q >= 10) */
    int n_edges;                    /* e-lines in the query */
} ora_plan;

/* Parse a query .g text and build the reference plan.  `enumerate_aut`:
 * run the reference's brute-force automorphism enumeration (needed for
 * last_sym/sym_count; exponential, so callers pass 0 for large symmetric
 * queries).  Returns an ORA_* exit code. */
int ora_query_plan(const char* text, size_t len, int enumerate_aut, ora_plan* out);

typedef struct {
    uint64_t count;                 /* embeddings found (after optional ref symmetry) */
    uint64_t rows_written;
    uint64_t partials[ORA_MAXQ];    /* |P_d|: partial matches with d+1 vertices */
    uint64_t lookups[ORA_MAXQ];     /* (vertex,label) list lookups made to extend depth d */
    uint64_t list_words[ORA_MAXQ];  /* sum of looked-up list lengths for depth d */
} ora_stats;

/* Enumerate embeddings with roots in [root_begin, root_end).
 *   ref_symmetry: apply the reference's lastSymmetry constraints (only when
 *                 sym_count > 1, like src/smsm.cu:1305-1319); the count is
 *                 then NOT multiplied (caller multiplies by sym_count).
 *   rows/rows_cap: optional table in reference column order.
 *   threads: worker threads (roots are claimed in chunks).
 *   limit: stop early (returning ORA_EXIT_LIMIT) once the search has
 *          visited more than `limit` nodes (partial matches and embeddings);
 *          0 = no limit.
 *   scan_limit: the same for the driver-list candidates the nodes scanned
 *          (a node whose lists are long does work without making nodes). */
int ora_match(const ora_graph* g, const ora_plan* p, int ref_symmetry,
              uint32_t root_begin, uint32_t root_end, int threads,
              uint32_t* rows, uint64_t rows_cap, uint64_t limit, uint64_t scan_limit, ora_stats* st);
/* ora_match with count_rule = 1: without a table, a last depth with a single
 * requirement is counted from its list (length minus the copies of the
 * vertices already matched) instead of being enumerated; the count is the
 * same (not part of the reference, which always enumerates). */
int ora_match_ex(const ora_graph* g, const ora_plan* p, int ref_symmetry,
                 uint32_t root_begin, uint32_t root_end, int threads,
                 uint32_t* rows, uint64_t rows_cap, uint64_t limit, uint64_t scan_limit, int count_rule,
                 ora_stats* st);

#ifdef __cplusplus
}
#endif
#endif
