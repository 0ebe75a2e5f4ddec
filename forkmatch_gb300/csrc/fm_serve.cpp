// fm_serve.cpp -- serving: a request loop over one resident graph.
//
// The reference runs one query per process (src/smsm.cu:1351-1393) on a slab
// it bump-allocates and never frees (src/trie.cuh:1029-1049).  A server keeps
// the graph resident and turns the context's slab into a pool of leases:
//
//   * admission: requests wait in arrival order; the head is admitted when an
//     idle slot exists and its lease -- level buffers sized by the estimated
//     partial matches of its widest level (at least one 32-parent chunk per
//     level for the graph's longest list, the kernels' hard minimum), plus a
//     table region in table mode -- fits the free pool (first fit);
//   * continuous batching: every slot is one host thread and one stream, so
//     admitted requests overlap on the device while later ones queue; a slot
//     that finds several count-mode requests at the head takes up to
//     max_batch of them into one shared launch sequence (fm_batch, no graph
//     capture, on scratch the slot owns: nothing is allocated per request);
//   * a lease that proves too small never changes a result: level buffers
//     defer and drain inside fm_match, a device table that truncated is
//     matched again with a lease of the exact size, and a level buffer below
//     one chunk is retried at twice the size.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fm_internal.h"
#include "fm_pool.h"

using namespace fm;

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint64_t kGranule = 2ull << 20;

uint64_t round_up(uint64_t x, uint64_t g) { return (x + g - 1) / g * g; }

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
    uint64_t ticket = 0;
    fm_query query;
    int32_t mode = FM_MODE_COUNT;
    uint32_t* host_rows = nullptr;
    uint64_t host_cap = 0;
    uint64_t level_rows = 0;        // estimated rows of the widest level
    uint64_t table_rows = 0;        // estimated embeddings (table mode)
    Clock::time_point t_submit, t_start;
    fm_serve_result res{};
};

struct Lease {
    uint64_t off = 0, bytes = 0;
    uint64_t soln_bytes = 0, table_bytes = 0;
};

// level columns of fm_match (rows with d entries at depths 2..q-1) and of a
// batch (d + 1 entries: the query id rides along)
uint64_t level_words(uint32_t q, bool batch) {
    uint64_t s = 0;
    for (uint32_t d = 2; d < q; d++) s += batch ? d + 1 : d;
    return s;
}

}  // namespace

struct fm_server {
    fm_context* ctx = nullptr;
    const fm_graph* graph = nullptr;
    fm_server_opts opts{};
    char* base = nullptr;           // lease pool
    fm::PoolAlloc pool;
    uint64_t min_rows = 0;          // one 32-parent chunk of the longest list, plus one bank
    struct Slot {
        fm_context* ctx = nullptr;
        BatchScratch scratch{};
    };
    std::vector<Slot> slots;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_ticket = 1;
    uint64_t submitted = 0, completed = 0, running = 0, batches = 0, embeddings = 0, limited = 0;
    bool stop = false;

    // Lease for a group of requests (one request, or count-mode requests
    // matched together).
    Lease lease_for(const std::vector<Request*>& group, uint64_t table_rows_override) const {
        Lease L;
        const bool batch = group.size() > 1;
        uint32_t maxq = 0;
        uint64_t rows = 0;
        for (const Request* r : group) {
            maxq = std::max(maxq, r->query.p.q);
            rows += r->level_rows;
        }
        const uint64_t words = level_words(maxq, batch);
        if (words) {
            const uint64_t want = std::max<uint64_t>(rows, min_rows) * 4 * words;
            const uint64_t hard = min_rows * 4 * words;
            L.soln_bytes = std::max(hard, std::min(std::max(want, opts.min_lease_bytes), opts.max_lease_bytes));
            L.soln_bytes = round_up(L.soln_bytes, kGranule);
        }
        if (!batch && group[0]->mode == FM_MODE_TABLE) {
            const Request* r = group[0];
            // the caller's buffer bounds the rows that can be returned: a
            // table of that size never needs a second run
            uint64_t trows = table_rows_override ? table_rows_override : r->host_rows ? r->host_cap : r->table_rows;
            if (r->host_rows) trows = std::min<uint64_t>(trows, r->host_cap);
            trows = std::max<uint64_t>(trows, 1);
            uint64_t tb = trows * 4ull * r->query.p.q;
            if (!table_rows_override) tb = std::min(tb, opts.max_lease_bytes);
            L.table_bytes = round_up(std::max<uint64_t>(tb, kGranule), kGranule);
        }
        L.bytes = std::max<uint64_t>(L.soln_bytes + L.table_bytes, kGranule);
        return L;
    }

    // Called with `mu` held: take the head request (and, when batching, the
    // count-mode requests right behind it) if its lease fits.
    bool admit(std::vector<Request*>& group, Lease& L) {
        while (!pending.empty()) {
            const int r = admit_head(group, L);
            if (r >= 0) return r == 1;
        }
        return false;
    }

    // 1: admitted; 0: the head must wait; -1: the head was rejected (try the next)
    int admit_head(std::vector<Request*>& group, Lease& L) {
        group.clear();
        group.push_back(pending.front());
        if (opts.max_batch > 1 && !opts.work_limit && group[0]->mode == FM_MODE_COUNT) {
            for (size_t i = 1; i < pending.size() && group.size() < opts.max_batch; i++) {
                if (pending[i]->mode != FM_MODE_COUNT) break;
                group.push_back(pending[i]);
            }
        }
        while (true) {
            L = lease_for(group, 0);
            if (pool.alloc(L.bytes, L.off)) break;
            if (group.size() > 1) {   // a smaller group may fit now
                group.pop_back();
                continue;
            }
            if (running) return 0;   // wait for leases to come back
            // the pool is idle and still too small: shrink the level part to
            // what is free (never below the hard minimum)
            const uint64_t largest = pool.largest();
            const uint64_t words = level_words(group[0]->query.p.q, false);
            const uint64_t hard = round_up(min_rows * 4 * words, kGranule);
            if (largest >= L.table_bytes + hard && L.soln_bytes > hard) {
                L.soln_bytes = (largest - L.table_bytes) / kGranule * kGranule;
                L.bytes = std::max<uint64_t>(L.soln_bytes + L.table_bytes, kGranule);
                if (pool.alloc(L.bytes, L.off)) break;
            }
            // cannot be served by this pool at all
            Request* r = group[0];
            pending.pop_front();
            r->t_start = Clock::now();
            r->res.status = FM_ERR_POOL;
            std::snprintf(r->res.error, sizeof(r->res.error), "the pool cannot hold this request's smallest lease");
            r->res.done = 1;
            r->res.latency_ms = r->res.queue_ms = ms_between(r->t_submit, r->t_start);
            completed++;
            cv_done.notify_all();
            group.clear();
            return -1;
        }
        for (size_t i = 0; i < group.size(); i++) pending.pop_front();
        return 1;
    }

    void run_single(Slot& slot, Request* r, Lease& L, std::unique_lock<std::mutex>& lk);
    void run_batch(Slot& slot, std::vector<Request*>& group, const Lease& L);
    void worker(size_t i);
};

namespace {

void set_regions(fm_context* c, char* base, const Lease& L) {
    char* p = base + L.off;
    context_set_regions(c, p, L.soln_bytes, (uint32_t*)(p + L.soln_bytes), L.table_bytes);
}

}  // namespace

// Runs with `mu` released; `lk` is taken only to swap leases on a retry.
void fm_server::run_single(Slot& slot, Request* r, Lease& L, std::unique_lock<std::mutex>& lk) {
    fm_result res;
    fm_status st = FM_OK;
    for (uint32_t attempt = 1;; attempt++) {
        set_regions(slot.ctx, base, L);
        fm_match_opts o;
        fm_match_opts_default(&o);
        o.mode = r->mode;
        o.host_rows = r->host_rows;
        o.host_rows_cap = r->host_cap;
        o.work_limit = opts.work_limit;
        // slots overlap on the GPU: a cooperative launch needs the whole GPU
        // resident at once, so served requests use level launches
        o.engine = FM_ENGINE_LEVELS;
        st = fm_match(slot.ctx, graph, &r->query, &o, &res);
        r->res.attempts = attempt;
        r->res.lease_bytes = L.bytes;
        Lease next;
        bool retry = false;
        if (st == FM_ERR_OUTPUT_OVERFLOW && r->host_rows && res.rows < std::min<uint64_t>(res.count, r->host_cap)) {
            // the device table truncated before the caller's buffer: match
            // again with a table of exactly the rows the caller can take
            std::vector<Request*> one{r};
            next = lease_for(one, std::min<uint64_t>(res.count, r->host_cap));
            next.soln_bytes = L.soln_bytes;
            next.bytes = next.soln_bytes + next.table_bytes;
            retry = true;
        } else if (st == FM_ERR_POOL && L.soln_bytes < pool.total() / 2) {
            next = L;
            next.soln_bytes = round_up(std::max<uint64_t>(2 * L.soln_bytes, kGranule), kGranule);
            next.bytes = next.soln_bytes + next.table_bytes;
            retry = true;
        }
        if (!retry || attempt >= 4) break;
        lk.lock();
        pool.release(L.off, L.bytes);
        cv_work.notify_all();
        bool ok = false;
        while (!(ok = pool.alloc(next.bytes, next.off))) {
            if (running <= 1 && pool.largest() < next.bytes) break;   // only this request is left
            cv_done.wait_for(lk, std::chrono::milliseconds(5));
        }
        if (!ok) {
            // keep the old lease slot accounting consistent: take back what fits
            if (!pool.alloc(L.bytes, L.off)) L.bytes = 0;
            lk.unlock();
            break;
        }
        L = next;
        lk.unlock();
    }
    // the caller's buffer took fewer rows than there are embeddings
    if (st == FM_OK && r->mode == FM_MODE_TABLE && r->host_rows && res.rows_copied < res.count) {
        set_error("host buffer smaller than the table; count is exact");
        st = FM_ERR_OUTPUT_OVERFLOW;
    }
    r->res.status = st;
    r->res.count = res.count;
    r->res.rows_copied = res.rows_copied;
    r->res.truncated = (st == FM_ERR_OUTPUT_OVERFLOW) ? 1 : 0;
    r->res.batch = 1;
}

void fm_server::run_batch(Slot& slot, std::vector<Request*>& group, const Lease& L) {
    set_regions(slot.ctx, base, L);
    std::vector<const fm_query*> qs;
    for (Request* r : group) qs.push_back(&r->query);
    fm_batch* b = nullptr;
    fm_status st = batch_create_scratch(slot.ctx, graph, qs.data(), (uint32_t)qs.size(), FM_MODE_COUNT, slot.scratch,
                                        &b);
    std::vector<uint64_t> counts(group.size(), 0);
    if (st == FM_OK) {
        batch_set_replay(b, false);
        st = fm_batch_run(b, counts.data(), nullptr);
        fm_batch_free(b);
    }
    for (size_t i = 0; i < group.size(); i++) {
        Request* r = group[i];
        r->res.status = st;
        r->res.count = st == FM_OK ? counts[i] : 0;
        r->res.batch = (uint32_t)group.size();
        r->res.attempts = 1;
        r->res.lease_bytes = L.bytes;
    }
}

void fm_server::worker(size_t i) {
    Slot& slot = slots[i];
    cudaSetDevice(ctx ? context_view(ctx).device : 0);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        std::vector<Request*> group;
        Lease L;
        while (true) {
            if (admit(group, L)) break;
            if (stop && pending.empty()) return;
            cv_work.wait(lk);
        }
        running += group.size();
        const Clock::time_point t0 = Clock::now();
        for (Request* r : group) r->t_start = t0;
        if (group.size() > 1) batches++;
        lk.unlock();
        if (group.size() == 1) run_single(slot, group[0], L, lk);
        else run_batch(slot, group, L);
        const Clock::time_point t1 = Clock::now();
        for (Request* r : group) {
            if (r->res.status != FM_OK) std::snprintf(r->res.error, sizeof(r->res.error), "%s", fm_last_error());
        }
        lk.lock();
        if (L.bytes) pool.release(L.off, L.bytes);
        running -= group.size();
        for (Request* r : group) {
            r->res.queue_ms = ms_between(r->t_submit, r->t_start);
            r->res.service_ms = ms_between(r->t_start, t1);
            r->res.latency_ms = ms_between(r->t_submit, t1);
            r->res.done = 1;
            completed++;
            if (r->res.status == FM_OK || r->res.status == FM_ERR_OUTPUT_OVERFLOW) embeddings += r->res.count;
            if (r->res.status == FM_ERR_LIMIT) limited++;
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" {

fm_status fm_server_create(fm_context* ctx, const fm_graph* g, const fm_server_opts* opts_in, fm_server** out) {
    if (!ctx || !g || !out) return FM_ERR_ARG;
    *out = nullptr;
    fm_server_opts o;
    if (opts_in) o = *opts_in;
    else std::memset(&o, 0, sizeof(o));
    if (o.slots == 0) o.slots = 4;
    if (o.slots > 64) o.slots = 64;
    if (o.max_batch == 0) o.max_batch = 1;
    if (o.max_batch > 4096) o.max_batch = 4096;
    const ContextView cv = context_view(ctx);
    if (g->g.device != cv.device) {
        set_error("graph and context live on different devices");
        return FM_ERR_ARG;
    }
    uint64_t slab_bytes = 0;
    char* slab = context_slab(ctx, &slab_bytes);
    const uint64_t misc_all = (uint64_t)o.slots * kContextMiscBytes;
    if (!slab || slab_bytes < misc_all + 64 * kGranule) {
        set_error("PREALLOC too small for the server's slots");
        return FM_ERR_POOL;
    }
    FM_CUDA(cudaSetDevice(cv.device));
    FM_CUDA(cudaStreamSynchronize(cv.stream));   // nothing of the context may still run on the slab
    if (!context_set_serving(ctx, true)) {
        set_error("the context already serves");
        return FM_ERR_ARG;
    }
    std::unique_ptr<fm_server, void (*)(fm_server*)> s(new fm_server(), fm_server_destroy);
    s->ctx = ctx;
    s->graph = g;
    // slot control regions at the top of the slab, the pool below
    const uint64_t pool_bytes = (slab_bytes - misc_all) / kGranule * kGranule;
    s->base = slab;
    s->pool.init(pool_bytes);
    if (o.max_lease_bytes == 0) o.max_lease_bytes = std::max<uint64_t>(pool_bytes / 4, kGranule);
    // The footprint model assumes independent e-lines and underestimates
    // skewed graphs badly, and a level buffer that is too small costs a
    // host-driven drain per refill; so by default every slot may hold half
    // of its even share of the pool, whatever the estimate says.
    if (o.min_lease_bytes == 0)
        o.min_lease_bytes = std::max<uint64_t>(256ull << 20, pool_bytes / (2ull * o.slots) / kGranule * kGranule);
    o.min_lease_bytes = std::min(o.min_lease_bytes, o.max_lease_bytes);
    s->opts = o;
    s->min_rows = (uint64_t)g->g.max_len * 32 + 32 + cv.bank_rows;
    for (uint32_t i = 0; i < o.slots; i++) {
        fm_server::Slot slot;
        fm_status st = context_create_view(ctx, slab + pool_bytes + (uint64_t)i * kContextMiscBytes, &slot.ctx);
        if (st != FM_OK) return st;
        slot.scratch.d_bytes = batch_scratch_bytes(o.max_batch, true);
        slot.scratch.h_bytes = batch_scratch_bytes(o.max_batch, false);
        cudaError_t e = cudaMalloc(&slot.scratch.d, slot.scratch.d_bytes);
        if (e == cudaSuccess) e = cudaHostAlloc(&slot.scratch.h, slot.scratch.h_bytes, cudaHostAllocDefault);
        s->slots.push_back(slot);
        if (e != cudaSuccess) return cuda_fail(e, "server slot scratch");
    }
    for (size_t i = 0; i < s->slots.size(); i++) s->workers.emplace_back([srv = s.get(), i] { srv->worker(i); });
    *out = s.release();
    return FM_OK;
}

fm_status fm_server_submit(fm_server* s, const fm_query* q, int32_t mode, uint32_t* host_rows, uint64_t host_rows_cap,
                           uint64_t* ticket) {
    if (!s || !q || !ticket || (mode != FM_MODE_COUNT && mode != FM_MODE_TABLE)) return FM_ERR_ARG;
    std::unique_ptr<Request> r(new Request());
    r->query = *q;
    r->mode = mode;
    r->host_rows = host_rows;
    r->host_cap = host_rows ? host_rows_cap : 0;
    double est[kMaxQ];
    estimate_level_rows(q->p, s->graph->g, est);
    double widest = 0;
    for (uint32_t d = 1; d + 1 < q->p.q; d++) widest = std::max(widest, est[d]);
    const double cap = 1e15;
    r->level_rows = (uint64_t)std::min(widest, cap);
    r->table_rows = q->p.q ? (uint64_t)std::min(est[q->p.q - 1], cap) : 0;
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        set_error("server is shutting down");
        return FM_ERR_ARG;
    }
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->pending.push_back(r.get());
    s->reqs[r->ticket] = std::move(r);
    s->submitted++;
    s->cv_work.notify_one();
    return FM_OK;
}

fm_status fm_server_poll(fm_server* s, uint64_t ticket, int32_t wait_ms, fm_serve_result* out) {
    if (!s || !out) return FM_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) {
        set_error("unknown ticket");
        return FM_ERR_ARG;
    }
    Request* r = it->second.get();
    if (!r->res.done && wait_ms != 0) {
        if (wait_ms < 0) s->cv_done.wait(lk, [&] { return r->res.done != 0; });
        else s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return r->res.done != 0; });
    }
    *out = r->res;
    return FM_OK;
}

fm_status fm_server_release(fm_server* s, uint64_t ticket) {
    if (!s) return FM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || !it->second->res.done) {
        set_error("unknown or unfinished ticket");
        return FM_ERR_ARG;
    }
    s->reqs.erase(it);
    return FM_OK;
}

fm_status fm_server_get_stats(fm_server* s, fm_server_stats* out) {
    if (!s || !out) return FM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->queued = s->pending.size();
    out->running = s->running;
    out->batches = s->batches;
    out->embeddings = s->embeddings;
    out->pool_bytes = s->pool.total();
    out->pool_free = s->pool.free_bytes();
    out->pool_peak_used = s->pool.peak();
    return FM_OK;
}

void fm_server_destroy(fm_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers)
        if (t.joinable()) t.join();
    for (auto& slot : s->slots) {
        if (slot.ctx) fm_context_destroy(slot.ctx);
        if (slot.scratch.d) cudaFree(slot.scratch.d);
        if (slot.scratch.h) cudaFreeHost(slot.scratch.h);
    }
    if (s->ctx) context_set_serving(s->ctx, false);
    delete s;
}

}  // extern "C"
