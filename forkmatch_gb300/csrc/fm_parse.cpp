// fm_parse.cpp -- .g text parsers and the query planner (host side).
//
// Data graphs: the reference reads the whole file on the host and parses it on
// the device (src/trie.cuh:1051-1222, line grammar src/trie.cuh:818-876).  Here
// the framing rules are the same (prefix "t # 0\n", trailer "t # -1" as the
// last six bytes, header "V E VL EL"), lines are parsed by all host threads in
// parallel, and malformed lines are reported instead of trapping.  Unlike the
// reference (whose 4-byte line-start windows never see the first content line,
// src/trie.cuh:829-834,1176-1178) every line is parsed, and files larger than
// 2 GiB are accepted (the reference's `int inputSize`, src/trie.cuh:1115).
//
// Queries: src/hostparser.cuh:286-508 (fileParse: degree-descending vertex
// order, src/hostparser.cuh:20-30) and src/ccsr.cuh:229-326,485-549 (matching
// order and requirements).  The automorphism count replaces the reference's
// brute-force enumeration (src/ccsr.cuh:383-465) with an orbit-stabiliser
// search, so large symmetric queries do not take exponential time.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>

#include "fm_internal.h"

namespace fm {

namespace {

inline bool parse_u32(const char*& p, const char* end, uint32_t& v) {
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

struct DataHeader {
    uint32_t V = 0, E = 0, VL = 0, EL = 0;
};

// Parses one body line starting at p; on success advances p past its '\n'.
// kind: 'v' or 'e'.  Returns false on a malformed line.
inline bool parse_line(const char*& p, const char* end, char& kind, uint32_t vals[3]) {
    if (p + 1 >= end) return false;
    kind = p[0];
    if ((kind != 'v' && kind != 'e') || p[1] != ' ') return false;
    p += 2;
    int nv = kind == 'e' ? 3 : 2;
    for (int k = 0; k < nv; k++) {
        if (!parse_u32(p, end, vals[k]) || p >= end) return false;
        char sep = (k == nv - 1) ? '\n' : ' ';
        if (*p != sep) return false;
        ++p;
    }
    return true;
}

}  // namespace

fm_status parse_data_text(const char* text, uint64_t len, EdgeArrays& out) {
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
        if (field > 3 || !parse_u32(p, end, h[field]) || p >= end) {
            set_error("malformed data graph header");
            return FM_ERR_DATA_HEADER;
        }
        if (*p == '\n') { ++p; break; }
        if (*p != ' ') { set_error("malformed data graph header"); return FM_ERR_DATA_HEADER; }
        ++p;
    }
    const uint32_t V = h[0];
    const uint64_t Ehdr = h[1];
    const uint32_t EL = h[3];
    const uint32_t L = std::min<uint32_t>(EL, FM_MAX_LABEL) + 1;   // labels > 255 are never matchable
    const char* body = p;
    const uint64_t blen = (uint64_t)(end - body);
    if (blen && body[blen - 1] != '\n') {
        set_error("last data line is not terminated by a newline before \"t # -1\"");
        return FM_ERR_DATA_LINE;
    }

    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    unsigned T = (unsigned)std::min<uint64_t>(std::min(hw, 64u), std::max<uint64_t>(1, blen >> 20));
    std::vector<const char*> cs(T + 1);
    cs[0] = body;
    cs[T] = end;
    for (unsigned t = 1; t < T; t++) {
        const char* q = body + blen * t / T;
        if (q < cs[t - 1]) q = cs[t - 1];
        if (q > body && q < end && q[-1] != '\n') {   // move to the next line start
            const char* nl = (const char*)std::memchr(q, '\n', (size_t)(end - q));
            q = nl ? nl + 1 : end;
        }
        cs[t] = q;
    }
    std::vector<uint64_t> cnt(T, 0);
    std::vector<const char*> bad(T, nullptr);
    auto count_pass = [&](unsigned t) {
        const char* s = cs[t];
        const char* e = cs[t + 1];
        uint64_t n = 0;
        char kind;
        uint32_t v[3];
        while (s < e) {
            const char* line = s;
            if (!parse_line(s, e, kind, v)) { bad[t] = line; break; }
            if (kind == 'v') {
                if (v[0] >= V) { bad[t] = line; break; }
                continue;
            }
            if (v[0] >= V || v[1] >= V || v[2] > EL) { bad[t] = line; break; }
            n += v[2] < L;
        }
        cnt[t] = n;
    };
    {
        std::vector<std::thread> th;
        for (unsigned t = 1; t < T; t++) th.emplace_back(count_pass, t);
        count_pass(0);
        for (auto& x : th) x.join();
    }
    for (unsigned t = 0; t < T; t++) {
        if (bad[t]) {
            const char* nl = (const char*)std::memchr(bad[t], '\n', (size_t)(end - bad[t]));
            std::string line(bad[t], nl ? (size_t)(nl - bad[t]) : std::min<size_t>(40, (size_t)(end - bad[t])));
            set_error("malformed or out-of-range data line: \"" + line.substr(0, 80) + "\"");
            return FM_ERR_DATA_LINE;
        }
    }
    std::vector<uint64_t> off(T + 1, 0);
    for (unsigned t = 0; t < T; t++) off[t + 1] = off[t] + cnt[t];
    if (off[T] > Ehdr) {
        set_error("more e-lines than the header's edge count");
        return FM_ERR_DATA_LINE;
    }
    out.V = V;
    out.L = L;
    out.src.resize(off[T]);
    out.dst.resize(off[T]);
    out.lab.resize(off[T]);
    auto fill_pass = [&](unsigned t) {
        const char* s = cs[t];
        const char* e = cs[t + 1];
        uint64_t i = off[t];
        char kind;
        uint32_t v[3];
        while (s < e) {
            parse_line(s, e, kind, v);
            if (kind == 'e' && v[2] < L) {
                out.src[i] = v[0];
                out.dst[i] = v[1];
                out.lab[i] = v[2];
                ++i;
            }
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < T; t++) th.emplace_back(fill_pass, t);
    fill_pass(0);
    for (auto& x : th) x.join();
    return FM_OK;
}

// ------------------------------------------------------------------ queries

namespace {

struct QEdge {
    uint32_t a, b, l;
};

struct LabelSet {   // set of labels of the e-lines a -> b
    uint64_t w[4] = {0, 0, 0, 0};
    void add(uint32_t l) { w[l >> 6] |= 1ull << (l & 63); }
    bool operator==(const LabelSet& o) const {
        return w[0] == o.w[0] && w[1] == o.w[1] && w[2] == o.w[2] && w[3] == o.w[3];
    }
};

// Is there an automorphism (a permutation preserving every labelled e-line set
// a -> b) that fixes 0..i-1 and sends i to u?
struct AutSearch {
    uint32_t q;
    LabelSet ls[kMaxQ][kMaxQ];
    uint32_t sig[kMaxQ];       // cheap invariant: out-degree * 64 + in-degree
    uint32_t f[kMaxQ];
    bool used[kMaxQ];
    uint64_t budget;

    bool consistent(uint32_t x, uint32_t y, uint32_t upto) const {
        if (sig[x] != sig[y]) return false;
        if (!(ls[x][x] == ls[y][y])) return false;
        for (uint32_t j = 0; j < upto; j++) {
            if (!(ls[x][j] == ls[y][f[j]]) || !(ls[j][x] == ls[f[j]][y])) return false;
        }
        return true;
    }
    bool rec(uint32_t d) {
        if (d == q) return true;
        if (budget == 0) return false;
        --budget;
        for (uint32_t y = 0; y < q; y++) {
            if (used[y] || !consistent(d, y, d)) continue;
            f[d] = y;
            used[y] = true;
            if (rec(d + 1)) return true;
            used[y] = false;
        }
        return false;
    }
    bool exists(uint32_t i, uint32_t u) {
        std::memset(used, 0, sizeof(used));
        for (uint32_t j = 0; j < i; j++) { f[j] = j; used[j] = true; }
        if (used[u] || !consistent(i, u, i)) return false;
        f[i] = u;
        used[u] = true;
        return rec(i + 1);
    }
};

uint64_t count_automorphisms(uint32_t q, const std::vector<QEdge>& es) {
    AutSearch s;
    std::memset(&s, 0, sizeof(s));
    s.q = q;
    for (const auto& e : es) {
        s.ls[e.a][e.b].add(e.l);
        s.sig[e.a] += 64;
        s.sig[e.b] += 1;
    }
    s.budget = 50'000'000;
    uint64_t total = 1;
    for (uint32_t i = 0; i < q; i++) {
        uint64_t orbit = 0;
        for (uint32_t u = 0; u < q; u++) orbit += s.exists(i, u) ? 1 : 0;
        if (s.budget == 0) return 0;
        if (orbit == 0) return 0;
        if (total > UINT64_MAX / orbit) return 0;   // does not fit: report "not computed"
        total *= orbit;
    }
    return total;
}

}  // namespace

fm_status compile_query_text(const char* text, uint64_t len, Plan& P) {
    P = Plan();
    const char* p = text;
    const char* end = text + len;
    auto bad = [](const char* why) {
        set_error(std::string("malformed query: ") + why);
        return FM_ERR_QUERY_FORMAT;
    };
    if (len < 6 || std::memcmp(p, "t # 0\n", 6) != 0) return bad("missing \"t # 0\\n\"");
    p += 6;
    uint32_t h[4] = {0, 0, 0, 0};
    for (int field = 0;; field++) {
        if (field > 3 || !parse_u32(p, end, h[field]) || p >= end) return bad("header");
        if (*p == '\n') { ++p; break; }
        if (*p != ' ') return bad("header");
        ++p;
    }
    const uint32_t q = h[0], Ehdr = h[1];
    if (q == 0) return bad("zero vertices");
    if (q > (uint32_t)kMaxQ) {
        set_error("query has more than 32 vertices");
        return FM_ERR_UNSUPPORTED;
    }
    std::vector<QEdge> es;
    uint32_t nv = 0;
    bool in_edges = false, ended = false;
    while (p < end) {
        if (end - p >= 6 && std::memcmp(p, "t # -1", 6) == 0) { ended = true; break; }
        char kind = *p;
        if (kind == 'e') in_edges = true;
        if (kind == 'v' && in_edges) return bad("vertex line after edge lines");
        uint32_t v[3];
        if (!parse_line(p, end, kind, v)) return bad("line");
        if (kind == 'v') { ++nv; continue; }
        if (v[0] >= q || v[1] >= q) return bad("edge endpoint out of range");
        if (v[2] > FM_MAX_LABEL) return bad("edge label above 255");
        if (es.size() >= 4096) {
            set_error("query has too many edges");
            return FM_ERR_UNSUPPORTED;
        }
        es.push_back({v[0], v[1], v[2]});
    }
    if (!ended) return bad("missing \"t # -1\"");
    if (nv < q || es.size() < Ehdr) {
        set_error("query has fewer vertex/edge lines than its header states");
        return FM_ERR_QUERY_MISSING;
    }
    P.q = q;
    P.e_lines = (uint32_t)es.size();

    // Local (CCSR) order: out-degree descending, then id ascending.
    uint32_t deg[kMaxQ] = {};
    for (const auto& e : es) deg[e.a]++;
    std::vector<uint32_t> ids(q);
    for (uint32_t i = 0; i < q; i++) ids[i] = i;
    std::sort(ids.begin(), ids.end(), [&](uint32_t x, uint32_t y) {
        return deg[x] != deg[y] ? deg[x] > deg[y] : x < y;
    });
    uint32_t loc[kMaxQ];
    for (uint32_t i = 0; i < q; i++) { P.inv[i] = ids[i]; loc[ids[i]] = i; }
    if (q >= 2) {
        for (uint32_t i = 0; i < q; i++) {
            if (deg[i] == 0) {
                set_error("query vertex without out-edges (disconnected query)");
                return FM_ERR_DISCONNECTED;
            }
        }
    }
    // Rows: (neighbour local, label) in e-line order, stable-sorted by neighbour.
    std::vector<std::vector<std::pair<uint32_t, uint32_t>>> row(q);
    for (const auto& e : es) row[loc[e.a]].push_back({loc[e.b], e.l});
    for (uint32_t v = 0; v < q; v++) {
        auto& r = row[v];
        std::stable_sort(r.begin(), r.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
        P.max_valency = std::max<uint32_t>(P.max_valency, (uint32_t)r.size());
        for (const auto& [m, l] : r) P.rows.push_back({v, m, l});
    }
    // Matching order: greedy, lowest local index on the frontier.
    int state[kMaxQ];
    for (uint32_t i = 0; i < q; i++) state[i] = -1;
    state[0] = 0;
    uint32_t total_req = 0;
    for (uint32_t depth = 0; depth < q; depth++) {
        int nw = -1;
        for (uint32_t i = 0; i < q; i++) {
            if (state[i] == 0 && nw < 0) { state[i] = 1; nw = (int)i; }
            else if (state[i] > 0) state[i]++;
        }
        if (nw < 0) {
            set_error("query is disconnected");
            return FM_ERR_DISCONNECTED;
        }
        P.order_local[depth] = (uint32_t)nw;
        struct R { uint32_t climb, l, refl; };
        std::vector<R> rs;
        for (const auto& [m, l] : row[nw]) {
            if (state[m] < 0) state[m] = 0;
            if (state[m] > 0) {
                uint32_t refl = l;
                for (const auto& [m2, l2] : row[m]) {
                    if (m2 == (uint32_t)nw) { refl = l2; break; }
                }
                rs.push_back({(uint32_t)(state[m] - 1), l, refl});
            }
        }
        std::stable_sort(rs.begin(), rs.end(), [](const R& x, const R& y) { return x.climb < y.climb; });
        if (!rs.empty() && rs[0].climb == 0) {
            set_error("query has a self loop");
            return FM_ERR_DISCONNECTED;
        }
        if (rs.size() > (size_t)kMaxQ || total_req + rs.size() > (size_t)kMaxReqTotal) {
            set_error("too many back edges at one depth");
            return FM_ERR_UNSUPPORTED;
        }
        if (depth > 0 && rs.empty()) {
            set_error("a depth has no back edge (the reference traps here)");
            return FM_ERR_UNSUPPORTED;
        }
        P.nreq[depth] = (uint32_t)rs.size();
        total_req += (uint32_t)rs.size();
        uint32_t pk = 0;
        for (size_t i = 0; i < rs.size(); i++) {
            P.req_climb[depth][i] = rs[i].climb;
            P.req_label[depth][i] = rs[i].l;
            P.req_refl[depth][i] = rs[i].refl;
        }
        for (size_t i = 0; i < rs.size(); i++) {
            pk = rs[i].climb;
            if (pk) break;
        }
        P.pk_dist[depth] = pk;
    }
    std::vector<QEdge> les;
    for (const auto& e : es) les.push_back({loc[e.a], loc[e.b], e.l});
    P.automorphisms = count_automorphisms(q, les);
    return FM_OK;
}

bool order_requirements(const Plan& P, const uint32_t* order, uint32_t nreq[kMaxQ],
                        uint32_t climb[kMaxQ][kMaxQ], uint32_t label[kMaxQ][kMaxQ]) {
    int depth_of[kMaxQ];
    for (uint32_t i = 0; i < P.q; i++) depth_of[i] = -1;
    for (uint32_t d = 0; d < P.q; d++) depth_of[order[d]] = (int)d;
    for (uint32_t d = 0; d < P.q; d++) {
        const uint32_t v = order[d];
        uint32_t n = 0;
        uint32_t c[kMaxQ], l[kMaxQ];
        for (const auto& e : P.rows) {       // rows are grouped by a, ordered by neighbour
            if (e.a != v || depth_of[e.b] < 0 || depth_of[e.b] >= (int)d) continue;
            if (n == (uint32_t)kMaxQ) return false;
            c[n] = d - (uint32_t)depth_of[e.b];
            l[n] = e.l;
            n++;
        }
        // stable sort by climb
        for (uint32_t i = 1; i < n; i++) {
            uint32_t cc = c[i], ll = l[i], j = i;
            while (j > 0 && c[j - 1] > cc) { c[j] = c[j - 1]; l[j] = l[j - 1]; j--; }
            c[j] = cc;
            l[j] = ll;
        }
        if (d > 0 && n == 0) return false;
        nreq[d] = n;
        for (uint32_t i = 0; i < n; i++) { climb[d][i] = c[i]; label[d][i] = l[i]; }
    }
    return true;
}

// Greedy order by estimated growth, over every start vertex.  Under a random
// graph model with the data graph's label frequencies, extending a partial
// match by a vertex with back e-lines of labels l1..lk yields about
//   min_i(E_li / V) * prod_{other i}(E_li / V^2)
// candidates: the shortest list drives, each further list filters.  Each step
// takes the vertex with the smallest factor (so cycles close as early as
// possible), ties broken by more back e-lines, larger degree, lower local
// index; the start with the smallest summed partial-match estimate wins, and
// ties keep the reference's start (local index 0 comes first).
void choose_order(const Plan& P, const DeviceGraph& g, uint32_t order[kMaxQ]) {
    const uint32_t q = P.q;
    for (uint32_t d = 0; d < q; d++) order[d] = P.order_local[d];
    if (q <= 2 || g.V == 0) return;
    const double V = (double)g.V;
    auto avg = [&](uint32_t l) {
        uint64_t c = l < g.label_count.size() ? g.label_count[l] : 0;
        return (double)c / V;
    };
    uint32_t deg[kMaxQ] = {};
    for (const auto& e : P.rows) deg[e.a]++;
    double best = -1;
    uint32_t cand[kMaxQ];
    for (uint32_t start = 0; start < q; start++) {
        bool matched[kMaxQ] = {};
        matched[start] = true;
        cand[0] = start;
        double card = V, cost = V;
        bool ok = true;
        for (uint32_t d = 1; d < q && ok; d++) {
            int pick = -1;
            double pf = 0;
            uint32_t pback = 0;
            for (uint32_t v = 0; v < q; v++) {
                if (matched[v]) continue;
                double mn = 1e300, prod = 1.0;
                uint32_t back = 0;
                for (const auto& e : P.rows) {
                    if (e.a != v || !matched[e.b]) continue;
                    double a = avg(e.l);
                    back++;
                    if (a < mn) {
                        if (mn < 1e299) prod *= mn / V;
                        mn = a;
                    } else {
                        prod *= a / V;
                    }
                }
                if (!back) continue;
                double f = mn * prod;
                bool better = pick < 0 || f < pf * (1 - 1e-12) ||
                              (f <= pf * (1 + 1e-12) && (back > pback || (back == pback && deg[v] > deg[pick])));
                if (better) {
                    pick = (int)v;
                    pf = f;
                    pback = back;
                }
            }
            if (pick < 0) { ok = false; break; }
            matched[pick] = true;
            cand[d] = (uint32_t)pick;
            card *= pf;
            cost += card;
        }
        if (!ok) continue;
        if (best < 0 || cost < best * (1 - 1e-9)) {
            best = cost;
            for (uint32_t d = 0; d < q; d++) order[d] = cand[d];
        }
    }
}

void estimate_level_rows(const Plan& P, const DeviceGraph& g, double est[kMaxQ]) {
    const uint32_t q = P.q;
    for (uint32_t d = 0; d < kMaxQ; d++) est[d] = 0;
    if (q == 0) return;
    uint32_t order[kMaxQ];
    choose_order(P, g, order);
    const double V = (double)g.V;
    auto avg = [&](uint32_t l) {
        uint64_t c = l < g.label_count.size() ? g.label_count[l] : 0;
        return V > 0 ? (double)c / V : 0.0;
    };
    bool matched[kMaxQ] = {};
    matched[order[0]] = true;
    double card = V;
    est[0] = card;
    for (uint32_t d = 1; d < q; d++) {
        const uint32_t v = order[d];
        double mn = 1e300, prod = 1.0;
        for (const auto& e : P.rows) {
            if (e.a != v || !matched[e.b]) continue;
            const double a = avg(e.l);
            if (a < mn) {
                if (mn < 1e299) prod *= mn / V;
                mn = a;
            } else {
                prod *= a / V;
            }
        }
        if (mn > 1e299) mn = 0;
        card *= mn * prod;
        est[d] = card;
        matched[v] = true;
    }
}

}  // namespace fm
