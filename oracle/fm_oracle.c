/*
 * fm_oracle.c -- CPU oracle for the ForkMatch hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see fm_oracle.h for what it restates and how it is
 * pinned).  Plain C11 + pthreads; builds with gcc on x86_64 and aarch64.
 */
#define _GNU_SOURCE
#include "fm_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

struct ora_graph {
    uint32_t V;
    uint32_t L;        /* label slots: labels 0..L-1 */
    uint64_t E;
    uint64_t* off;     /* L*V + 1 offsets into nbr, key = label*V + src */
    uint32_t* nbr;     /* destinations, sorted ascending within a (label, src) segment */
};

uint32_t ora_graph_vertices(const ora_graph* g) { return g->V; }
uint64_t ora_graph_edges(const ora_graph* g) { return g->E; }
uint32_t ora_graph_labels(const ora_graph* g) { return g->L; }

uint64_t ora_graph_list(const ora_graph* g, uint32_t label, uint32_t v, const uint32_t** ptr) {
    if (label >= g->L || v >= g->V) { *ptr = g->nbr; return 0; }
    uint64_t k = (uint64_t)label * g->V + v;
    *ptr = g->nbr + g->off[k];
    return g->off[k + 1] - g->off[k];
}

uint32_t ora_graph_sources(const ora_graph* g, uint32_t label) {
    uint32_t n = 0;
    if (label >= g->L) return 0;
    for (uint32_t v = 0; v < g->V; v++) {
        uint64_t k = (uint64_t)label * g->V + v;
        n += g->off[k + 1] != g->off[k];
    }
    return n;
}

void ora_graph_free(ora_graph* g) {
    if (!g) return;
    free(g->off);
    free(g->nbr);
    free(g);
}

/* Sorted (label, src, dst) order of src/trie.cuh:89-115, built with two
 * stable counting passes: by dst, then by (label, src). */
int ora_graph_from_edges(uint32_t V, uint32_t n_labels, uint64_t E,
                         const uint32_t* src, const uint32_t* dst,
                         const uint32_t* label, ora_graph** out) {
    *out = NULL;
    for (uint64_t i = 0; i < E; i++) {
        if (src[i] >= V || dst[i] >= V || label[i] >= n_labels) return ORA_EXIT_DATA_LINE;
    }
    ora_graph* g = (ora_graph*)calloc(1, sizeof(ora_graph));
    if (!g) return ORA_EXIT_DATA_LINE;
    g->V = V;
    g->L = n_labels;
    g->E = E;
    uint64_t K = (uint64_t)n_labels * V;
    g->off = (uint64_t*)calloc(K + 1, sizeof(uint64_t));
    g->nbr = (uint32_t*)malloc((E ? E : 1) * sizeof(uint32_t));
    uint64_t* cnt = (uint64_t*)calloc((uint64_t)V + 1, sizeof(uint64_t));
    uint64_t* perm = (uint64_t*)malloc((E ? E : 1) * sizeof(uint64_t));
    if (!g->off || !g->nbr || !cnt || !perm) {
        free(cnt); free(perm); ora_graph_free(g); return ORA_EXIT_DATA_LINE;
    }
    /* pass 1: stable order by dst */
    for (uint64_t i = 0; i < E; i++) cnt[dst[i] + 1]++;
    for (uint64_t v = 0; v < V; v++) cnt[v + 1] += cnt[v];
    for (uint64_t i = 0; i < E; i++) perm[cnt[dst[i]]++] = i;
    free(cnt);
    /* pass 2: stable order by key = label*V + src */
    for (uint64_t i = 0; i < E; i++) g->off[(uint64_t)label[i] * V + src[i] + 1]++;
    for (uint64_t k = 0; k < K; k++) g->off[k + 1] += g->off[k];
    uint64_t* cur = (uint64_t*)malloc((K ? K : 1) * sizeof(uint64_t));
    if (!cur) { free(perm); ora_graph_free(g); return ORA_EXIT_DATA_LINE; }
    memcpy(cur, g->off, K * sizeof(uint64_t));
    for (uint64_t j = 0; j < E; j++) {
        uint64_t i = perm[j];
        uint64_t k = (uint64_t)label[i] * V + src[i];
        g->nbr[cur[k]++] = dst[i];
    }
    free(cur);
    free(perm);
    *out = g;
    return ORA_OK;
}

/* ---- data .g text: src/trie.cuh:1075-1097 (framing, header),
 *      src/trie.cuh:838-873 (line grammar; SAFEPARSE) ---- */

static int parse_u32(const char** pp, const char* end, uint32_t* v) {
    const char* p = *pp;
    uint64_t acc = 0;
    int digits = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        acc = acc * 10 + (uint64_t)(*p - '0');
        if (acc > 0xffffffffull) return 0;
        p++;
        digits++;
    }
    if (!digits) return 0;
    *v = (uint32_t)acc;
    *pp = p;
    return 1;
}

int ora_graph_parse(const char* text, size_t len, ora_graph** out) {
    *out = NULL;
    if (len < 6 || memcmp(text, "t # 0\n", 6) != 0) return ORA_EXIT_DATA_HEADER0;
    if (len < 12 || memcmp(text + len - 6, "t # -1", 6) != 0) return ORA_EXIT_DATA_TRAILER;
    /* header: up to four space-separated integers ending in '\n' */
    uint32_t h[4] = {0, 0, 0, 0};
    const char* p = text + 6;
    const char* end = text + len - 6;
    int field = 0;
    for (;;) {
        if (p >= end) return ORA_EXIT_DATA_HEADER;
        if (!parse_u32(&p, end, &h[field])) return ORA_EXIT_DATA_HEADER;
        if (p >= end) return ORA_EXIT_DATA_HEADER;
        if (*p == '\n') { p++; break; }
        if (*p != ' ' || field == 3) return ORA_EXIT_DATA_HEADER;
        p++;
        field++;
    }
    uint32_t V = h[0];
    uint64_t Ehdr = h[1];
    uint32_t EL = h[3];
    /* body: lines "v id label" / "e src dst label", each ending in '\n' */
    uint64_t cap = Ehdr ? Ehdr : 16, n = 0;
    uint32_t* s = (uint32_t*)malloc(cap * sizeof(uint32_t));
    uint32_t* d = (uint32_t*)malloc(cap * sizeof(uint32_t));
    uint32_t* l = (uint32_t*)malloc(cap * sizeof(uint32_t));
    int rc = ORA_OK;
    while (p < end && rc == ORA_OK) {
        char kind = *p;
        if ((kind != 'v' && kind != 'e') || p + 1 >= end || p[1] != ' ') { rc = ORA_EXIT_DATA_LINE; break; }
        p += 2;
        uint32_t vals[3];
        int nv = kind == 'e' ? 3 : 2;
        for (int k = 0; k < nv; k++) {
            if (!parse_u32(&p, end, &vals[k]) || p >= end) { rc = ORA_EXIT_DATA_LINE; break; }
            char sep = (k == nv - 1) ? '\n' : ' ';
            if (*p != sep) { rc = ORA_EXIT_DATA_LINE; break; }
            p++;
        }
        if (rc != ORA_OK) break;
        if (kind == 'v') {
            if (vals[0] >= V) rc = ORA_EXIT_DATA_LINE;
            continue;
        }
        if (vals[0] >= V || vals[1] >= V || vals[2] > EL || n >= Ehdr) { rc = ORA_EXIT_DATA_LINE; break; }
        s[n] = vals[0]; d[n] = vals[1]; l[n] = vals[2]; n++;
    }
    if (rc == ORA_OK) rc = ora_graph_from_edges(V, EL + 1, n, s, d, l, out);
    free(s); free(d); free(l);
    return rc;
}

/* ---- query .g text and planner ---- */

typedef struct { int nbr, label; } qent;

static int cmp_order(const void* a, const void* b) {
    const int* x = (const int*)a;  /* [deg, id] */
    const int* y = (const int*)b;
    if (x[0] != y[0]) return y[0] - x[0];   /* degree descending */
    return x[1] - y[1];                     /* then id ascending */
}

typedef struct {
    int q;
    int deg[ORA_MAXQ];
    qent row[ORA_MAXQ][ORA_MAXQ * 4];       /* local rows, by local neighbour index */
} qgraph;

static int row_has(const qgraph* G, int v, int nbr, int label) {
    for (int i = 0; i < G->deg[v]; i++)
        if (G->row[v][i].nbr == nbr && G->row[v][i].label == label) return 1;
    return 0;
}

/* Reference queryMatch (src/ccsr.cuh:383-465) over local indices. */
typedef struct {
    const qgraph* G;
    int f[ORA_MAXQ];
    int used[ORA_MAXQ];
    int* auts;        /* n x q */
    uint64_t n, cap;
    int overflow;
} autctx;

static void aut_rec(autctx* c, int D) {
    const qgraph* G = c->G;
    if (D == G->q) {
        if (c->n == c->cap) {
            uint64_t nc = c->cap ? c->cap * 2 : 64;
            if (nc > (1ull << 24)) { c->overflow = 1; return; }
            c->auts = (int*)realloc(c->auts, nc * G->q * sizeof(int));
            c->cap = nc;
        }
        memcpy(c->auts + c->n * G->q, c->f, G->q * sizeof(int));
        c->n++;
        return;
    }
    for (int n = 0; n < G->q && !c->overflow; n++) {
        if (c->used[n]) continue;
        int ok = 1;
        for (int i = 0; i < G->deg[D] && ok; i++) {
            int m = G->row[D][i].nbr;
            if (m < D && !row_has(G, n, c->f[m], G->row[D][i].label)) ok = 0;
        }
        if (!ok) continue;
        c->f[D] = n;
        c->used[n] = 1;
        aut_rec(c, D + 1);
        c->used[n] = 0;
    }
}

int ora_query_plan(const char* text, size_t len, int enumerate_aut, ora_plan* P) {
    memset(P, 0, sizeof(*P));
    const char* p = text;
    const char* end = text + len;
    if (len < 6 || memcmp(p, "t # 0\n", 6) != 0) return ORA_EXIT_QUERY_INVALID;
    p += 6;
    uint32_t h[4] = {0, 0, 0, 0};
    int field = 0;
    for (;;) {
        if (!parse_u32(&p, end, &h[field]) || p >= end) return ORA_EXIT_QUERY_INVALID;
        if (*p == '\n') { p++; break; }
        if (*p != ' ' || field == 3) return ORA_EXIT_QUERY_INVALID;
        p++;
        field++;
    }
    uint32_t q = h[0], Ehdr = h[1];
    if (q == 0 || q > ORA_MAXQ) return ORA_EXIT_QUERY_INVALID;
    int es[ORA_MAXQ * ORA_MAXQ * 4][3];
    uint32_t ne = 0, nvx = 0;
    int in_edges = 0, ended = 0;
    while (p < end) {
        if (end - p >= 6 && memcmp(p, "t # -1", 6) == 0) { ended = 1; break; }
        char kind = *p;
        if (kind == 'e') in_edges = 1;
        if ((kind != 'v' && kind != 'e') || (kind == 'v' && in_edges) || p + 1 >= end || p[1] != ' ')
            return ORA_EXIT_QUERY_INVALID;
        p += 2;
        uint32_t vals[3];
        int nv = kind == 'e' ? 3 : 2;
        for (int k = 0; k < nv; k++) {
            if (!parse_u32(&p, end, &vals[k]) || p >= end) return ORA_EXIT_QUERY_INVALID;
            char sep = (k == nv - 1) ? '\n' : ' ';
            if (*p != sep) return ORA_EXIT_QUERY_INVALID;
            p++;
        }
        if (kind == 'v') { nvx++; continue; }
        if (vals[0] >= q || vals[1] >= q || vals[2] > 255 || ne >= sizeof(es) / sizeof(es[0]))
            return ORA_EXIT_QUERY_INVALID;
        es[ne][0] = (int)vals[0]; es[ne][1] = (int)vals[1]; es[ne][2] = (int)vals[2];
        ne++;
    }
    if (!ended) return ORA_EXIT_QUERY_INVALID;
    if (nvx < q || ne < Ehdr) return ORA_EXIT_QUERY_MISSING_DATA;
    P->q = (int)q;
    P->n_edges = (int)ne;

    /* degree-descending order (OrderPair, src/hostparser.cuh:20-30,420) */
    int deg[ORA_MAXQ] = {0};
    for (uint32_t i = 0; i < ne; i++) deg[es[i][0]]++;
    int ord[ORA_MAXQ][2];
    for (uint32_t i = 0; i < q; i++) { ord[i][0] = deg[i]; ord[i][1] = (int)i; }
    qsort(ord, q, sizeof(ord[0]), cmp_order);
    int loc[ORA_MAXQ];
    for (uint32_t i = 0; i < q; i++) { P->inv[i] = ord[i][1]; loc[ord[i][1]] = (int)i; }
    if (q >= 2) {
        for (uint32_t i = 0; i < q; i++)
            if (deg[i] == 0) return ORA_EXIT_PLAN;      /* vertex without a CCSR row */
    }
    qgraph G;
    memset(&G, 0, sizeof(G));
    G.q = (int)q;
    for (uint32_t i = 0; i < ne; i++) {
        int a = loc[es[i][0]];
        if (G.deg[a] >= ORA_MAXQ * 4) return ORA_EXIT_QUERY_INVALID;
        G.row[a][G.deg[a]].nbr = loc[es[i][1]];
        G.row[a][G.deg[a]].label = es[i][2];
        G.deg[a]++;
    }
    /* per-row order by neighbour (src/hostparser.cuh:480-493); stable insertion sort */
    int maxv = 0;
    for (uint32_t v = 0; v < q; v++) {
        for (int i = 1; i < G.deg[v]; i++) {
            qent t = G.row[v][i];
            int j = i - 1;
            while (j >= 0 && G.row[v][j].nbr > t.nbr) { G.row[v][j + 1] = G.row[v][j]; j--; }
            G.row[v][j + 1] = t;
        }
        if (G.deg[v] > maxv) maxv = G.deg[v];
    }
    P->max_valency = maxv;

    /* matching order and requirements (src/ccsr.cuh:229-326, 520-549) */
    int state[ORA_MAXQ];
    for (uint32_t i = 0; i < q; i++) state[i] = -1;
    state[0] = 0;
    for (uint32_t depth = 0; depth < q; depth++) {
        int nw = -1;
        for (uint32_t i = 0; i < q; i++) {
            if (state[i] == 0 && nw < 0) { state[i] = 1; nw = (int)i; }
            else if (state[i] > 0) state[i]++;
        }
        if (nw < 0) return ORA_EXIT_PLAN;
        P->order[depth] = nw;
        int n = 0;
        int climb[ORA_MAXQ * 4], lab[ORA_MAXQ * 4], refl[ORA_MAXQ * 4];
        for (int i = 0; i < G.deg[nw]; i++) {
            int m = G.row[nw][i].nbr;
            if (state[m] < 0) state[m] = 0;
            if (state[m] > 0) {
                int r = G.row[nw][i].label;
                for (int j = 0; j < G.deg[m]; j++)
                    if (G.row[m][j].nbr == nw) { r = G.row[m][j].label; break; }
                climb[n] = state[m] - 1;
                lab[n] = G.row[nw][i].label;
                refl[n] = r;
                n++;
            }
        }
        /* sort by climb (stable) */
        for (int i = 1; i < n; i++) {
            int c = climb[i], a = lab[i], b = refl[i], j = i - 1;
            while (j >= 0 && climb[j] > c) { climb[j + 1] = climb[j]; lab[j + 1] = lab[j]; refl[j + 1] = refl[j]; j--; }
            climb[j + 1] = c; lab[j + 1] = a; refl[j + 1] = b;
        }
        if (n > ORA_MAXQ) return ORA_EXIT_PLAN;
        P->nreq[depth] = n;
        int pk = 0;
        for (int i = 0; i < n; i++) {
            P->req_climb[depth][i] = climb[i];
            P->req_label[depth][i] = lab[i];
            P->req_refl[depth][i] = refl[i];
        }
        for (int i = 0; i < n; i++) {   /* first non-zero climb (src/ccsr.cuh:302-308) */
            pk = climb[i];
            if (pk) break;
        }
        P->pk_dist[depth] = pk;
        if (n && climb[0] == 0) return ORA_EXIT_PLAN;   /* self loop: src/ccsr.cuh:719-725 */
    }
    for (uint32_t d = 1; d < q; d++)
        if (P->nreq[d] == 0) return ORA_EXIT_PLAN;          /* reference traps in isoLoop */
    for (uint32_t i = 0; i < q; i++) P->ref_mapping[i] = P->order[q - 1 - i];

    /* symmetry (src/ccsr.cuh:487-507, 553-673) */
    P->sym_count = 1;
    P->aut_count = 0;
    if (!enumerate_aut) return ORA_OK;
    if (q >= 20) return ORA_EXIT_NO_IDENTITY;
    autctx A;
    memset(&A, 0, sizeof(A));
    A.G = &G;
    for (uint32_t i = 0; i < q && !A.overflow; i++) {
        A.f[0] = (int)i;
        A.used[i] = 1;
        aut_rec(&A, 1);
        A.used[i] = 0;
    }
    if (A.overflow) { free(A.auts); return ORA_EXIT_PLAN; }
    P->aut_count = A.n;
    P->sym_count = q >= 10 ? 1 : A.n;
    int ident = -1;
    for (uint64_t a = 0; a < A.n; a++) {
        int ok = 1;
        for (uint32_t i = 0; i < q; i++) if (A.auts[a * q + i] != (int)i) { ok = 0; break; }
        if (ok) ident = (int)a;
    }
    if (ident < 0) { free(A.auts); return ORA_EXIT_NO_IDENTITY; }
    int rev[ORA_MAXQ];
    for (uint32_t i = 0; i < q; i++) rev[P->ref_mapping[i]] = (int)i;
    uint32_t groups[ORA_MAXQ];
    memset(groups, 0, sizeof(groups));
    for (uint32_t pdx = 0; pdx < q; pdx++) {
        for (uint64_t a = 0; a < A.n; a++) {
            if ((int)a == ident) continue;
            const int* s = A.auts + a * q;
            int b = s[pdx];
            if (b == (int)pdx || b > (int)pdx) continue;
            if (s[b] != (int)pdx) continue;
            int agree = 1;
            for (uint32_t i = 0; i < pdx; i++)
                if ((int)i != b && s[i] != (int)i) { agree = 0; break; }
            if (!agree) continue;
            int left = rev[pdx], right = rev[b];
            groups[left] |= 1u << right;
            groups[right] |= 1u << left;
        }
    }
    for (int i = (int)q - 1; i >= 0; i--) {
        int d = (int)q - 1 - i;
        P->last_sym[d] = 0;
        for (int i2 = i + 1; i2 < (int)q; i2++) {
            if (groups[i] & (1u << i2)) { P->last_sym[d] = i2 - i; break; }
        }
    }
    free(A.auts);
    return ORA_OK;
}

/* ---- matcher ---- */

typedef struct {
    const ora_graph* g;
    const ora_plan* p;
    int ref_sym;
    uint32_t root_begin, root_end;
    uint64_t next_root;          /* atomic */
    uint32_t* rows;
    uint64_t rows_cap;
    uint64_t rows_next;          /* atomic */
    uint64_t limit;              /* stop after this many search nodes (0 = none) */
    uint64_t seen;               /* atomic, in steps of 4096 */
    uint64_t scan_limit;         /* stop after this many driver-list candidates (0 = none) */
    uint64_t scanned;            /* atomic */
    int aborted;                 /* atomic */
    int count_rule;              /* count the last depth from its list when it has one requirement */
    pthread_mutex_t mu;
    ora_stats total;
} mctx;

typedef struct {
    mctx* m;
    uint32_t f[ORA_MAXQ];
    ora_stats st;
    uint64_t nodes;              /* search-tree nodes visited (for the limit) */
    uint64_t scans;              /* candidates not yet added to m->scanned */
} wctx;

static uint64_t lower_b(const uint32_t* a, uint64_t n, uint32_t x) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) { uint64_t mid = (lo + hi) >> 1; if (a[mid] < x) lo = mid + 1; else hi = mid; }
    return lo;
}

static void dfs(wctx* w, int d) {
    const ora_plan* P = w->m->p;
    const ora_graph* g = w->m->g;
    int q = P->q;
    if (__atomic_load_n(&w->m->aborted, __ATOMIC_RELAXED)) return;
    if (w->m->limit && (++w->nodes & 4095) == 0) {
        /* the limit bounds the search: every node of the search tree counts */
        uint64_t s = __atomic_add_fetch(&w->m->seen, 4096, __ATOMIC_RELAXED);
        if (s > w->m->limit) __atomic_store_n(&w->m->aborted, 1, __ATOMIC_RELAXED);
    }
    if (d == q) {
        w->st.count++;
        if (w->m->rows) {
            uint64_t idx = __atomic_fetch_add(&w->m->rows_next, 1, __ATOMIC_RELAXED);
            if (idx < w->m->rows_cap) {
                uint32_t* r = w->m->rows + idx * (uint64_t)q;
                for (int c = 0; c < q; c++) r[c] = w->f[q - 1 - c];
            }
        }
        return;
    }
    int k = P->nreq[d];
    const uint32_t* lp[ORA_MAXQ];
    uint64_t ln[ORA_MAXQ];
    int drv = 0;
    for (int i = 0; i < k; i++) {
        uint32_t anc = w->f[d - P->req_climb[d][i]];
        ln[i] = ora_graph_list(g, (uint32_t)P->req_label[d][i], anc, &lp[i]);
        w->st.lookups[d]++;
        w->st.list_words[d] += ln[i];
        if (ln[i] < ln[drv]) drv = i;
    }
    if (w->m->scan_limit && k) {
        /* the scan limit bounds the work a node does on its driver list */
        w->scans += ln[drv];
        if (w->scans >= 4096) {
            uint64_t s = __atomic_add_fetch(&w->m->scanned, w->scans, __ATOMIC_RELAXED);
            w->scans = 0;
            if (s > w->m->scan_limit) {
                __atomic_store_n(&w->m->aborted, 1, __ATOMIC_RELAXED);
                return;
            }
        }
    }
    int sym = (w->m->ref_sym && P->sym_count > 1) ? P->last_sym[d] : 0;
    uint32_t bound = sym ? w->f[d - sym] : 0;
    if (w->m->count_rule && d == q - 1 && k == 1 && !sym && !w->m->rows) {
        /* Count rule: with one requirement, the last vertex can be any entry
         * of the list (duplicates included) except the vertices already
         * matched, so the extensions are the list length minus the copies of
         * each matched vertex in it.  Same count as enumerating them. */
        uint64_t c = ln[0];
        for (int a = 0; a < d; a++) {
            uint64_t lo = lower_b(lp[0], ln[0], w->f[a]);
            while (lo < ln[0] && lp[0][lo] == w->f[a]) { c--; lo++; }
        }
        w->st.partials[d] += c;
        w->st.count += c;
        return;
    }
    uint64_t j = 0;
    while (j < ln[drv]) {
        uint32_t x = lp[drv][j];
        uint64_t mult = 1;
        while (j + mult < ln[drv] && lp[drv][j + mult] == x) mult++;
        j += mult;
        for (int i = 0; i < k && mult; i++) {
            if (i == drv) continue;
            uint64_t lo = lower_b(lp[i], ln[i], x);
            uint64_t c = 0;
            while (lo + c < ln[i] && lp[i][lo + c] == x) c++;
            if (c < mult) mult = c;
        }
        if (!mult) continue;
        int ok = 1;
        for (int a = 0; a < d; a++) if (w->f[a] == x) { ok = 0; break; }
        if (ok && sym && !(x < bound)) ok = 0;
        if (!ok) continue;
        for (uint64_t r = 0; r < mult; r++) {
            w->f[d] = x;
            w->st.partials[d]++;
            dfs(w, d + 1);
        }
    }
}

static void* worker(void* arg) {
    wctx* w = (wctx*)arg;
    mctx* m = w->m;
    const ora_plan* P = m->p;
    const uint64_t chunk = 16;
    for (;;) {
        uint64_t b = __atomic_fetch_add(&m->next_root, chunk, __ATOMIC_RELAXED);
        if (b >= m->root_end || __atomic_load_n(&m->aborted, __ATOMIC_RELAXED)) break;
        uint64_t e = b + chunk < m->root_end ? b + chunk : m->root_end;
        for (uint64_t v = b; v < e; v++) {
            if (P->q >= 2) {
                /* isoInit keeps v iff the depth-1 list is non-empty (src/smsm.cu:835) */
                const uint32_t* lst;
                if (!ora_graph_list(m->g, (uint32_t)P->req_label[1][0], (uint32_t)v, &lst)) continue;
            }
            w->f[0] = (uint32_t)v;
            w->st.partials[0]++;
            dfs(w, 1);
        }
    }
    pthread_mutex_lock(&m->mu);
    m->total.count += w->st.count;
    for (int d = 0; d < ORA_MAXQ; d++) {
        m->total.partials[d] += w->st.partials[d];
        m->total.lookups[d] += w->st.lookups[d];
        m->total.list_words[d] += w->st.list_words[d];
    }
    pthread_mutex_unlock(&m->mu);
    return NULL;
}

int ora_match(const ora_graph* g, const ora_plan* p, int ref_symmetry,
              uint32_t root_begin, uint32_t root_end, int threads,
              uint32_t* rows, uint64_t rows_cap, uint64_t limit, uint64_t scan_limit, ora_stats* st) {
    return ora_match_ex(g, p, ref_symmetry, root_begin, root_end, threads, rows, rows_cap, limit, scan_limit, 0,
                        st);
}

int ora_match_ex(const ora_graph* g, const ora_plan* p, int ref_symmetry,
                 uint32_t root_begin, uint32_t root_end, int threads,
                 uint32_t* rows, uint64_t rows_cap, uint64_t limit, uint64_t scan_limit, int count_rule,
                 ora_stats* st) {
    mctx m;
    memset(&m, 0, sizeof(m));
    m.g = g; m.p = p; m.ref_sym = ref_symmetry;
    m.count_rule = count_rule;
    if (root_end > g->V) root_end = g->V;
    m.root_begin = root_begin; m.root_end = root_end;
    m.next_root = root_begin;
    m.rows = rows; m.rows_cap = rows_cap;
    m.limit = limit;
    m.scan_limit = scan_limit;
    pthread_mutex_init(&m.mu, NULL);
    if (threads < 1) threads = 1;
    if (threads > 512) threads = 512;
    wctx* ws = (wctx*)calloc((size_t)threads, sizeof(wctx));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    for (int t = 0; t < threads; t++) ws[t].m = &m;
    for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, worker, &ws[t]);
    worker(&ws[0]);
    for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
    m.total.rows_written = rows ? (m.rows_next < rows_cap ? m.rows_next : rows_cap) : 0;
    *st = m.total;
    free(ws);
    free(th);
    pthread_mutex_destroy(&m.mu);
    return m.aborted ? ORA_EXIT_LIMIT : ORA_OK;
}
