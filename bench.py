"""Benchmark: embeddings/sec of batched matching (512 queries in shared
launches replayed as a CUDA graph, the queries whose work fills the GPU alone
matched alone inside the run, as the autotuner picks) beside the plain form
(one fm_match per query), on the batched workload, with full uint32 embedding
tables for the table queries and u64 counts for the count-only ones.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --workload plain_at_scale|plain_small|serving|skew|ingest

Workload (forkmatch_gb300.workloads, default "batched"): R-MAT(0.57, 0.19,
0.19, 0.05) with 2^22 vertices and 64M distinct undirected edges (128M
e-lines), 64 edge labels, 8 vertex labels; 512 queries of 4-16 vertices
recorded with their exact counts in tests/golden/workload_batched.json.  One
step matches all 512 queries.  The other workloads: plain_at_scale (R-MAT
2^20, 16M edges, 16 queries of 8 vertices, one at a time), serving (Poisson
arrivals against a resident 2^24-vertex graph, p50/p99), skew (count-only
stress on a Chung-Lu graph with work limits), ingest (the batched graph as
>2 GiB .g text).

ours       value: batched embeddings/s, device-timed (CUDA events on the
           library's stream) with the graph resident and the queries compiled;
           "plain" beside it, timed the same way.  e2e: through the C ABI from
           host inputs every step (query texts compiled, batch created and run,
           every table copied into pinned host memory).  cpu_baseline: the CPU
           port on whole sampled queries over the full root range.
reference  the reference has no CPU matcher, so its arm is the project's CPU
           port of its algorithm (oracle/) on all host threads: a fixed sample
           of whole queries, each over the full root range, spread over the K
           timed steps.

Multi-GPU (torchrun): the batched workload splits its queries over the ranks
by recorded cost; plain_at_scale splits the roots into contiguous ranges of
equal estimated work (degree squared).  Counts are summed as int64 and the
time is the maximum over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

GB = 1 << 30
E2E_STEPS = 5
METRIC = "embeddings/sec"
UNIT = "embeddings/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "plain_at_scale", "plain_small", "serving", "skew", "ingest"])
    ap.add_argument("--ncu-step", action="store_true",
                    help="run one untimed step with small knobs (SOLN 2 GiB, OUTPUT 4.5 GiB) for ncu captures")
    ap.add_argument("--queries", default="all", help="with --ncu-step: comma-separated query indices")
    ap.add_argument("--ncu-scale", type=int, default=0,
                    help="with --ncu-step --workload batched: match on an R-MAT graph of 2^N vertices and 16 * 2^N "
                         "edges with the workload's generator parameters instead of the full graph (counts "
                         "are not checked)")
    # serving workload
    ap.add_argument("--serving-scale", type=int, default=24, help="log2 vertices (edges scale along)")
    ap.add_argument("--serving-queries", type=int, default=128)
    ap.add_argument("--serving-seconds", type=float, default=3.0)
    ap.add_argument("--serving-requests", type=int, default=20000)
    ap.add_argument("--rates", default="100,1000,3000,10000")
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--max-batch", type=int, default=32)
    ap.add_argument("--pool-gb", type=int, default=120)
    ap.add_argument("--serving-max-ms", type=float, default=20.0, help="latency bound of the query screen")
    ap.add_argument("--skew-limit", type=int, default=1 << 36, help="work limit per query of the skew workload")
    ap.add_argument("--soln-gb", type=float, default=24.0, help="SOLN_PREALLOC of the plain-at-scale context, GiB")
    return ap.parse_args()


def match_alg_bytes(r, qi, count_only):
    """Algorithmic bytes of one match from its per-level work counters: per
    depth, 16 B per (vertex, label) record lookup, 4 B per word of the
    looked-up lists and 8 B per partial match stored in a level buffer; 4q B
    per table row.  The last depth stores no partial matches (its rows are
    table rows, or only counted).  A count-only last depth with one back edge
    is charged its lookups only (the count rule: one record per parent, the
    parent's vertices tested against it), and the depth before it stores
    nothing when the match counted from there (pre-count)."""
    q = qi.q
    b = 0
    for d in range(1, q):
        lv = r.level[d]
        rule = count_only and d == q - 1 and qi.nreq[d] == 1
        stored = d < q - 1 and not (r.pre_counted and d == q - 2)
        b += 16 * lv.lookups + (0 if rule else 4 * lv.list_words) + (8 * lv.produced if stored else 0)
    return b + (0 if count_only else 4 * q * r.count)


def run_ncu_step(args):
    """One step of the workload with small knobs, for ncu captures (prints the
    total count; every count is checked against the recorded one).  With
    --workload ingest: the device parse and graph build of a 2^20-vertex,
    8M-edge R-MAT graph as .g text (about 311 MB)."""
    import forkmatch_gb300 as fm
    if args.workload == "ingest":
        from forkmatch_gb300 import synth as S
        G = S.rmat(20, 8_000_000, 13, 64)
        text = G.to_g_text()
        ctx = fm.Context(prealloc_bytes=1 * GB, soln_prealloc_bytes=256 << 20, output_prealloc_bytes=256 << 20)
        g = fm.Graph.from_text(ctx, text)
        inf = g.info()
        print("ncu step ok", len(text), inf.edges, inf.segments)
        g.close()
        ctx.close()
        return 0
    if args.ncu_scale and args.workload == "batched":
        from forkmatch_gb300 import synth as S
        from forkmatch_gb300 import workloads as W
        wl = W.load_workload("batched")
        p = W.BATCHED
        G = S.rmat(args.ncu_scale, 16 << args.ncu_scale, p["seed"], p["n_elabels"])
        src, dst, lab = G.directed()
        same = False
    else:
        wl, G, (src, dst, lab), same, _ = load_workload(args.workload)
    pick = None if args.queries == "all" else {int(x) for x in args.queries.split(",")}
    # the table region only as large as the picked table queries need
    need = sum(q["count"] * query_vertices(q) * 4 for i, q in enumerate(wl["queries"])
               if (pick is None or i in pick) and not is_count_only(q))
    out_bytes = min(int(4.5 * GB), ((need + (64 << 20)) >> 20) << 20)
    ctx = fm.Context(prealloc_bytes=2 * GB + out_bytes + (128 << 20), soln_prealloc_bytes=2 * GB,
                     output_prealloc_bytes=out_bytes, bank_rows=1 << 12)
    g = fm.Graph.from_edges(ctx, G.V, G.n_elabels + 1, src, dst, lab)
    if args.workload == "batched":
        # one batch (table mode, as in the benchmark) of the picked queries;
        # their algorithmic bytes come first from the plain kernels' counters
        # (k_expand launches, outside a k_bexpand capture filter)
        idx = [i for i in range(len(wl["queries"])) if pick is None or i in pick]
        qs = [fm.Query.from_text(wl["queries"][i]["text"].encode()) for i in idx]
        counted = [is_count_only(wl["queries"][i]) for i in idx]
        alg = 0
        for q, c_only in zip(qs, counted):
            qi = q.info()
            r = fm.match(ctx, g, q, mode=fm.MODE_COUNT if c_only else fm.MODE_TABLE, profile=True)
            alg += match_alg_bytes(r, qi, c_only)
        b = fm.Batch(ctx, g, qs, mode=fm.MODE_TABLE)
        for i, c_only in enumerate(counted):
            if c_only:
                b.set_query_mode(i, fm.MODE_COUNT)
        counts, _ = b.run()
        if same and counts != [wl["queries"][i]["count"] for i in idx]:
            raise SystemExit("count mismatch in the batch")
        print("ncu step ok", sum(counts), "algorithmic_bytes", alg)
        return 0
    tot = 0
    for i, qm in enumerate(wl["queries"]):
        if pick is not None and i not in pick:
            continue
        r = fm.match(ctx, g, fm.Query.from_text(qm["text"].encode()), mode=fm.MODE_TABLE)
        if same and r.count != qm["count"]:
            raise SystemExit("count mismatch on query %d: %d != %d" % (i, r.count, qm["count"]))
        tot += r.count
    print("ncu step ok", tot)
    return 0


def profiled_traffic():
    """DRAM bytes per level launch from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_expand_plain_at_scale.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_level_launch:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.lines = []
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_workload(name):
    from forkmatch_gb300 import workloads as W
    wl = W.load_workload(name)
    t = time.time()
    G = {"plain_at_scale": W.plain_at_scale_graph, "batched": W.batched_graph}[name]()
    src, dst, lab = G.directed()
    same = W.edge_hash(src, dst, lab) == wl["edge_sha256"]
    return wl, G, (src, dst, lab), same, time.time() - t


def root_ranges(src, V, world):
    """Contiguous root ranges of equal estimated work, one per rank."""
    from forkmatch_gb300 import shard
    return shard.root_ranges_weighted(shard.root_work_weights(src, V), world)


# ------------------------------------------------------------------ reference arm

def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=20).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# Queries of the CPU samples: whole queries over the full root range (per-root
# work is heavy-tailed on R-MAT, so a root prefix is not representative).
# Every 10th query of the batched mix (52 queries, every size 4-16 and every
# shape) for the reference arm, every 32nd (16 queries) for cpu_baseline; all
# 16 queries of the plain-at-scale workload.
REF_EVERY = {"batched": 10, "plain_at_scale": 1}
CPU_EVERY = {"batched": 32, "plain_at_scale": 1}


def oracle_sample(wl, every):
    return [i for i in range(len(wl["queries"])) if i % every == 0]


def query_vertices(qm):
    """Vertices of a recorded query (the first field of its .g header line)."""
    return int(qm["text"].split("\n")[1].split()[0])


def is_count_only(qm):
    """Queries recorded as count only (their tables have 10^9 rows or more)."""
    return qm.get("mode", "table") == "count"


def run_reference(args, rank, world):
    """The reference arm: the project's CPU port of the reference's algorithm
    (the reference has no CPU matcher of its own) on all host threads.  The
    sample's queries are spread over the K timed steps (step s takes every
    K-th query of the sample from position s), each over the full root range,
    so the K steps together match every sampled query exactly once."""
    if rank != 0:
        return 0
    from oracle import oracle as O
    wl, G, (src, dst, lab), same, gen_s = load_workload(args.workload)
    og = O.Graph.from_edges(G.V, G.n_elabels + 1, src, dst, lab)
    del src, dst, lab
    threads = os.cpu_count() or 1
    sample = oracle_sample(wl, REF_EVERY.get(args.workload, 1))
    plans = {i: O.plan(wl["queries"][i]["text"].encode(), enumerate_aut=0) for i in sample}
    steps = max(1, args.steps)
    parts = [sample[s::steps] for s in range(steps)]
    warm = min(sample, key=lambda i: wl["queries"][i]["count"])

    for _ in range(args.warmup):
        O.match(og, plans[warm], threads=threads, count_rule=is_count_only(wl["queries"][warm]))
    t0 = time.perf_counter()
    total = 0
    counts = {}
    for part in parts:
        for i in part:
            c = O.match(og, plans[i], threads=threads, count_rule=is_count_only(wl["queries"][i]))[0]
            counts[i] = c
            total += c
    el = time.perf_counter() - t0
    value = total / el
    exact = all(counts[i] == wl["queries"][i]["count"] for i in sample) if same else None
    desc = ("%d of the %d queries (every %d-th), each over the full root range, split over the %d timed steps; "
            "%d embeddings in %.1f s on %d threads of %s" % (len(sample), len(wl["queries"]),
                                                             REF_EVERY.get(args.workload, 1), steps, total, el,
                                                             threads, cpu_model()))
    config = batched_config(wl, G, same) if args.workload == "batched" else workload_config(wl, G, same)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el / steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic", "config": config, "counts_equal_recorded": exact,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc,
                             "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def workload_config(wl, G, same):
    return {"workload": wl["workload"], "graph": "R-MAT(0.57,0.19,0.19,0.05) 2^20 vertices, 16M undirected edges "
            "(32M e-lines), 32 edge labels, Zipf(1.2) vertex labels over 4", "vertices": G.V, "e_lines": wl["E"],
            "queries": len(wl["queries"]), "query_vertices": 8,
            "query_mix": "8 random-walk dense (density>=0.5) + 8 random-walk sparse (0.40<=density<0.50; "
                         "spanning trees have ~1e16 embeddings and are not enumerable)",
            "mode": "plain: one query per launch sequence, full uint32 embedding tables",
            "graph_matches_recorded_hash": same,
            "l2": "inputs larger than L2: resident graph 1.6 GB (records, lists, bitmaps) vs 129 MB L2, 10.6 GB of table rows written per step; no flush between steps"}


# ------------------------------------------------------------------ our arm

def run_ours(args, rank, world, local):
    import torch
    import forkmatch_gb300 as fm
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl, G, (src, dst, lab), same, gen_s = load_workload(args.workload)
    queries_meta = wl["queries"]
    max_count = max(q["count"] for q in queries_meta)
    out_bytes = ((int(max_count * 8 * 4 * 1.05) + (64 << 20)) >> 20) << 20
    # the slab beyond SOLN + OUTPUT is the pool of the served e2e path
    ctx = fm.Context(prealloc_bytes=64 * GB, soln_prealloc_bytes=int(args.soln_gb * GB),
                     output_prealloc_bytes=out_bytes, bank_rows=1 << 16, device=local)
    t = time.time()
    g = fm.Graph.from_edges(ctx, G.V, G.n_elabels + 1, src, dst, lab)
    build_s = time.time() - t
    ginfo = g.info()
    queries = [fm.Query.from_text(q["text"].encode()) for q in queries_meta]
    qinfo = [q.info() for q in queries]
    rb, re_ = root_ranges(src, G.V, world)[rank]
    stream = torch.cuda.ExternalStream(ctx.stream)

    def step(collect=None, profile=False):
        c = 0
        launches = 0
        for i, q in enumerate(queries):
            r = fm.match(ctx, g, q, mode=fm.MODE_TABLE, roots=(rb, re_), profile=profile)
            c += r.count
            launches += r.launches
            if collect is not None:
                collect.append(r)
        return c, launches

    # verification (untimed): exact counts at full size + row validity on a sample
    results = []
    total, _ = step(collect=results)
    counts = [r.count for r in results]
    bitexact = None
    if world == 1:
        bitexact = counts == [q["count"] for q in queries_meta] if same else None
    rows_ok = verify_rows(ctx, g, queries, qinfo, (src, dst, lab), roots=(rb, re_))

    # roofline pass (untimed): per-launch CUDA events inside the library
    prof = []
    step(collect=prof, profile=True)
    alg_bytes = 0
    kern_ms = 0.0
    n_launch = 0
    for r, qi in zip(prof, qinfo):
        for d in range(1, qi.q):
            kern_ms += r.level[d].kernel_ms
            n_launch += r.level[d].launches
        alg_bytes += match_alg_bytes(r, qi, False)
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (kern_ms / 1000.0) / 1e9 if kern_ms > 0 else None

    for _ in range(args.warmup):
        step()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local) if rank == 0 else None
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    total = 0
    launches = 0
    for _ in range(args.steps):
        c, l = step()
        total += c
        launches += l
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    ms = e0.elapsed_time(e1)
    if world > 1:
        torch.distributed.barrier()

    # end to end through the C ABI: host query text in, table out to pinned host
    # memory.  Two ways out: the kernels write the rows straight into the
    # pinned buffer over the host link (host_direct), or the table is built in
    # HBM and copied with one cudaMemcpyAsync.  Both are timed; e2e reports the
    # faster, "e2e_paths" both.
    pinned = fm.PinnedRows(max(counts) + 1, 8)
    texts = [q["text"].encode() for q in queries_meta]

    def e2e_step(direct):
        c = h2d = d2h = 0
        for tx in texts:
            q = fm.Query.from_text(tx)
            r = fm.match(ctx, g, q, mode=fm.MODE_TABLE, roots=(rb, re_), host_rows=pinned, host_direct=direct)
            c += r.count
            h2d += r.h2d_bytes + len(tx)
            d2h += r.d2h_bytes
            q.close()
        return c, h2d, d2h

    e2e_paths = {}
    for name, direct in (("host_direct", True), ("device_then_copy", False)):
        e2e_step(direct)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        tot_e = 0
        for _ in range(args.steps):
            c, hb, db = e2e_step(direct)
            tot_e += c
        el = time.perf_counter() - w0
        e2e_paths[name] = {"value": tot_e / el, "ms_per_step": 1000 * el / args.steps,
                           "h2d_bytes_per_step": hb, "d2h_bytes_per_step": db, "total": tot_e, "seconds": el}

    # served: the queries as table requests to a server (fm_server_*) with
    # three slots, so one request's table copy to the host overlaps the next
    # one's matching; every table lands in its own slice of one pinned buffer
    if world == 1:
        qw = [c * qi.q for c, qi in zip(counts, qinfo)]
        offs = np.concatenate([[0], np.cumsum(qw)]).astype(np.int64)
        host = fm.PinnedRows(int(offs[-1]) + 1, 1)
        views = [host.array[offs[i]:offs[i + 1]] for i in range(len(texts))]
        srv = fm.Server(ctx, g, slots=3, min_lease_bytes=8 * GB, max_lease_bytes=16 * GB)

        def e2e_served():
            tickets = []
            for tx, view in zip(texts, views):
                q = fm.Query.from_text(tx)
                tickets.append(srv.submit(q, mode=fm.MODE_TABLE, host_rows=view))
                q.close()
            c = d2h = 0
            for t, qi in zip(tickets, qinfo):
                r = srv.poll(t)
                if r.status != fm.FM_OK:
                    raise RuntimeError("served request failed with status %d: %s" % (r.status, r.error.decode()))
                c += r.count
                d2h += r.rows_copied * qi.q * 4
                srv.release(t)
            return c, sum(len(tx) for tx in texts), d2h

        try:
            e2e_served()
            w0 = time.perf_counter()
            tot_e = 0
            for _ in range(args.steps):
                c, hb, db = e2e_served()
                tot_e += c
            el = time.perf_counter() - w0
        finally:
            srv.close()
        e2e_paths["served_overlap"] = {"value": tot_e / el, "ms_per_step": 1000 * el / args.steps,
                                       "h2d_bytes_per_step": hb, "d2h_bytes_per_step": db, "total": tot_e,
                                       "seconds": el}
    best = max(e2e_paths, key=lambda k: e2e_paths[k]["value"])
    e_total, e2e_s = e2e_paths[best]["total"], e2e_paths[best]["seconds"]
    h2d, d2h = e2e_paths[best]["h2d_bytes_per_step"], e2e_paths[best]["d2h_bytes_per_step"]

    value = total / (ms / 1000.0)
    e2e_value = e_total / e2e_s
    if world > 1:
        (total, e_total), (ms, e2e_s) = allreduce_counts_and_times([total, e_total], [ms, e2e_s])
        value = total / (ms / 1000.0)
        e2e_value = e_total / e2e_s
    if rank != 0:
        return 0
    cpu = cpu_baseline(wl, G, (src, dst, lab), "plain_at_scale") if world == 1 else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generators)",
            "config": workload_config(wl, G, same),
            "embeddings_per_step": total / args.steps,
            "bitexact_counts": bitexact, "rows_valid_sample": rows_ok,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": profiled_traffic(),
                         "traffic_source": "profiles/k_expand_plain_at_scale.md (DRAM read+write per level launch)",
                         "kernel": "k_expand (all levels)", "peak_kind": peak_kind,
                         "algorithmic_bytes_per_step": alg_bytes, "kernel_ms_per_step": kern_ms,
                         "launches_per_step": n_launch,
                         "avg_launch_ms": kern_ms / max(1, n_launch)},
            "cpu_baseline": cpu,
            "e2e_paths": {k: {kk: vv for kk, vv in v.items() if kk not in ("total", "seconds")}
                          for k, v in e2e_paths.items()},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": best,
                    "ms_per_step": 1000 * e2e_s / args.steps},
            # every level launch is two kernels of ours: the main pass and the heavy pass
            "gpu_launches": 2 * launches, "clocks": clocks,
            "graph": {"build_ms": ginfo.build_ms, "device_bytes": ginfo.device_bytes, "max_list": ginfo.max_list,
                      "segments": ginfo.segments, "long_segments": ginfo.long_segments,
                      "generate_s": gen_s, "load_s": build_s}}
    print(json.dumps(line), flush=True)
    return 0


def batched_config(wl, G, same):
    from collections import Counter
    shapes = Counter(q["shape"] + (" (count only)" if is_count_only(q) else "") for q in wl["queries"])
    sizes = Counter(q["k"] for q in wl["queries"])
    return {"workload": "batched", "graph": "R-MAT(0.57,0.19,0.19,0.05) 2^22 vertices, 64M undirected edges "
            "(128M e-lines), 64 edge labels, 8 vertex labels uniform", "vertices": G.V, "e_lines": wl["E"],
            "queries": len(wl["queries"]), "query_vertices": "4-16 (%d to %d per size)" % (min(sizes.values()),
                                                                                      max(sizes.values())),
            "query_mix": dict(shapes),
            "excluded_shapes": sorted({"%s%d" % (x["shape"], x["k"]) for x in wl["excluded"]}),
            "screening": "table queries: kept when the oracle finishes within 2^27 search nodes with count <= "
                         "2^22; count-only queries: 4-vertex paths and stars pinned by exact closed forms, "
                         "5-vertex paths by the oracle with the count rule; larger paths, stars and cycles are "
                         "excluded with GPU time estimates (their slots hold walk subgraphs)",
            "mode": "batched: shared level launches (or one persistent cooperative launch) for all queries, "
                    "replayed as a CUDA graph; the autotuner picks the queries matched alone inside the run (those "
                    "whose work fills the GPU by itself: single-query engine, whole level memory), the engine, split "
                    "granularity, grid and level-buffer size; per-query uint64 counts + uint32 tables (count-only "
                    "queries: counts). plain: one fm_match per query",
            "graph_matches_recorded_hash": same,
            "l2": "inputs larger than L2: resident graph 5.7 GB vs 129 MB L2; no flush between steps"}


def batched_traffic(alg_shared, alg_alone):
    """DRAM bytes of one batch run: the ncu summary's DRAM bytes per
    algorithmic byte (captured on a smaller batch of the same queries) times
    this run's algorithmic bytes, separately for the queries in the shared
    launches (batch kernels) and the queries matched alone (single-query
    kernels)."""
    p = os.path.join(ROOT, "profiles", "k_bexpand_batched.md")
    ratio = {}
    try:
        for line in open(p):
            for key in ("traffic_bytes_per_algorithmic_byte", "traffic_bytes_per_algorithmic_byte_single"):
                if line.startswith(key + ":"):
                    ratio[key] = float(line.split(":")[1])
    except (OSError, ValueError):
        return None
    if len(ratio) < 2:
        return None
    return int(alg_shared * ratio["traffic_bytes_per_algorithmic_byte"] +
               alg_alone * ratio["traffic_bytes_per_algorithmic_byte_single"])


def allreduce_counts_and_times(counts, times):
    """Sum integer counts (int64, exact) and take the maximum of times over ranks."""
    import torch
    import torch.distributed as dist
    c = torch.tensor([int(x) for x in counts], dtype=torch.int64, device="cuda")
    t = torch.tensor([float(x) for x in times], dtype=torch.float64, device="cuda")
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [int(x) for x in c.cpu().tolist()], [float(x) for x in t.cpu().tolist()]


def run_batched(args, rank, world, local):
    """Batched vs plain on the 512-query workload.  Under torchrun the queries
    are split over the ranks by their recorded CPU cost (each rank matches
    whole queries against its own replica of the graph); counts are summed as
    int64 and times are the maximum over ranks."""
    import torch
    import forkmatch_gb300 as fm
    from forkmatch_gb300 import shard
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl, G, (src, dst, lab), same, gen_s = load_workload("batched")
    meta_all = wl["queries"]
    if world > 1:
        mine = shard.split_queries([q["oracle_seconds"] for q in meta_all], world)[rank]
    else:
        mine = list(range(len(meta_all)))
    meta = [meta_all[i] for i in mine]
    rec = [q["count"] for q in meta]
    counted = [is_count_only(q) for q in meta]
    modes = [fm.MODE_COUNT if c else fm.MODE_TABLE for c in counted]
    table_words = sum(q["count"] * q["k"] for q, c in zip(meta, counted) if not c)
    out_bytes = ((table_words * 4 + (256 << 20)) >> 20) << 20
    # one shared level buffer per depth holds every query's partial matches
    ctx = fm.Context(prealloc_bytes=128 * GB + out_bytes + (128 << 20), soln_prealloc_bytes=128 * GB,
                     output_prealloc_bytes=out_bytes, bank_rows=1 << 16, device=local)
    t = time.time()
    g = fm.Graph.from_edges(ctx, G.V, G.n_elabels + 1, src, dst, lab)
    build_s = time.time() - t
    queries = [fm.Query.from_text(q["text"].encode()) for q in meta]
    qinfo = [q.info() for q in queries]
    stream = torch.cuda.ExternalStream(ctx.stream)

    def plain_step(collect=None, profile=False):
        c = launches = 0
        for q, mode in zip(queries, modes):
            r = fm.match(ctx, g, q, mode=mode, profile=profile)
            c += r.count
            launches += r.launches
            if collect is not None:
                collect.append(r)
        return c, launches

    # verification (untimed): plain counts, sampled rows of the plain tables
    res = []
    plain_step(collect=res)
    plain_counts = [r.count for r in res]
    rng = np.random.default_rng(7)
    tabled = [i for i in range(len(meta)) if not counted[i]]
    sample = sorted(rng.choice(tabled, size=min(24, len(tabled)), replace=False).tolist())
    plain_rows = {}
    for i in sample:
        cnt, rows, _ = fm.match_table(ctx, g, queries[i], max_rows=max(1, rec[i]))
        plain_rows[i] = rows[np.lexsort(rows.T[::-1])] if len(rows) else rows

    # roofline numerator: the algorithmic bytes of every query (same matching
    # order in both forms), from the plain form's per-level counters
    prof = []
    plain_step(collect=prof, profile=True)
    alg_each = [match_alg_bytes(r, qi, c_only) for r, qi, c_only in zip(prof, qinfo, counted)]
    alg_bytes = sum(alg_each)

    b = fm.Batch(ctx, g, queries, mode=fm.MODE_TABLE)
    for i, c_only in enumerate(counted):
        if c_only:
            b.set_query_mode(i, fm.MODE_COUNT)
    b.run()
    tune = b.tune()
    counts, st = b.run()
    batch_ok = counts == rec if same else None
    plain_ok = plain_counts == rec if same else None
    rows_ok = True
    for i in sample:
        br = b.rows(i, rec[i])
        br = br[np.lexsort(br.T[::-1])] if len(br) else br
        if br.shape != plain_rows[i].shape or not np.array_equal(br, plain_rows[i]):
            rows_ok = False

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        tot = launches = 0
        for _ in range(steps):
            c, l = fn()
            tot += c
            launches += l
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return e0.elapsed_time(e1), tot, launches

    def batch_step():
        c, s = b.run()
        return sum(c), s.launches

    sampler = ClockSampler(local) if rank == 0 else None
    b_ms, b_tot, b_launch = timed(batch_step, args.steps)
    clocks = sampler.stop() if sampler else None
    p_ms, p_tot, p_launch = timed(plain_step, args.steps)

    # end to end through the C ABI, every step: the query texts compiled, the
    # batch created (plans uploaded, table regions sized by a counting run, the
    # level sequence captured), run, and every table copied to pinned host
    # memory with one copy
    host = fm.PinnedRows(table_words + 1, 1)
    texts = [q["text"].encode() for q in meta]

    # a later batch of the same queries reuses the tuner's choices that are
    # per query or per engine (the queries matched alone, the engine)
    solo_idx = b.solo()
    alg_alone = sum(alg_each[i] for i in solo_idx)

    def e2e_fresh():
        qs = [fm.Query.from_text(tx) for tx in texts]
        bb = fm.Batch(ctx, g, qs, mode=fm.MODE_TABLE)
        bb.set_engine(fm.ENGINE_PERSISTENT if st.persistent else fm.ENGINE_LEVELS)
        for i in solo_idx:
            bb.set_solo(i)
        for i, c_only in enumerate(counted):
            if c_only:
                bb.set_query_mode(i, fm.MODE_COUNT)
        c, _ = bb.run()
        words, _ = bb.copy_tables(host)
        bb.close()
        for q in qs:
            q.close()
        return sum(c), words * 4

    def e2e_replay():
        c, _ = b.run()
        words, _ = b.copy_tables(host)
        return sum(c), words * 4

    # (at most E2E_STEPS steps per path: a fresh batch costs a counting run,
    # a table run, graph captures and the 7 GB copy, several seconds a step)
    e2e_steps = max(1, min(args.steps, E2E_STEPS))
    e2e_paths = {}
    for name, fn in (("fresh_batch", e2e_fresh), ("replay", e2e_replay)):
        fn()
        if world > 1:
            torch.distributed.barrier()
        w0 = time.perf_counter()
        tot = 0
        for _ in range(e2e_steps):
            c, d2h = fn()
            tot += c
        el = time.perf_counter() - w0
        if world > 1:
            (tot,), (el,) = allreduce_counts_and_times([tot], [el])
        h2d = sum(len(tx) for tx in texts) if name == "fresh_batch" else 0
        e2e_paths[name] = {"value": tot / el, "ms_per_step": 1000 * el / e2e_steps, "steps": e2e_steps,
                           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    if world > 1:
        (b_tot, p_tot, alg_bytes, b_launch), (b_ms, p_ms) = allreduce_counts_and_times(
            [b_tot, p_tot, alg_bytes, b_launch], [b_ms, p_ms])
    if rank != 0:
        return 0
    e2e = dict(e2e_paths["fresh_batch"], unit=UNIT, path="fresh_batch")
    value = b_tot / (b_ms / 1000.0)
    plain_value = p_tot / (p_ms / 1000.0)
    peak, peak_kind = measured_peak_hbm()
    run_ms = b_ms / args.steps
    achieved = alg_bytes / (run_ms / 1000.0) / 1e9
    cpu = cpu_baseline(wl, G, (src, dst, lab), "batched") if world == 1 else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": run_ms, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generators)",
            "config": batched_config(wl, G, same),
            "embeddings_per_step": b_tot / args.steps,
            "embeddings_per_step_by_mode": {
                "table_queries": sum(c for c, co in zip(rec, counted) if not co),
                "count_only_queries": sum(c for c, co in zip(rec, counted) if co)},
            "plain": {"value": plain_value, "ms_per_step": p_ms / args.steps, "launches_per_step":
                      p_launch / args.steps},
            "batched_over_plain": value / plain_value,
            "bitexact_counts": {"batched": batch_ok, "plain": plain_ok},
            "rows_equal_sample": {"queries": len(sample), "equal": rows_ok},
            "tuned": {"engine": "persistent" if st.persistent else "levels",
                      "piece_shift": tune.piece_shift, "grid_quarters": tune.grid_quarters,
                      "level_rows": tune.level_rows, "weighted_levels": bool(st.weighted_levels),
                      "persistent": bool(st.persistent), "graph": bool(st.graph),
                      "batched_queries": st.batched_queries, "single_queries": st.single_queries,
                      "solo_queries": st.solo_queries},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": batched_traffic(alg_bytes / max(1, world) - alg_alone, alg_alone),
                         "kernel": "one batch run: k_bexpand + k_bexpand_heavy for the shared launches (k_bpersist "
                                   "when the tuner picks the persistent engine), k_expand + k_expand_heavy for the "
                                   "queries matched alone (the dominant one: the pre-count level of the 5-vertex "
                                   "count-only paths)",
                         "peak_kind": peak_kind, "algorithmic_bytes_per_step": alg_bytes,
                         "traffic_source": "profiles/k_bexpand_batched.md (DRAM bytes per algorithmic byte of "
                                           "the batch kernels and of the single-query kernels, captured on every "
                                           "32nd query at 2^20 vertices, applied to this run's shared and alone "
                                           "queries)",
                         "note": "achieved = algorithmic bytes of all queries / device time of one batch run"},
            "cpu_baseline": cpu,
            "e2e_paths": e2e_paths, "e2e": e2e,
            "gpu_launches": b_launch, "clocks": clocks,
            "graph": {"generate_s": gen_s, "load_s": build_s, "device_bytes": g.info().device_bytes}}
    print(json.dumps(line), flush=True)
    return 0


def run_serving(args, rank, world, local):
    """Request loop on the serving workload: Poisson arrivals at swept rates
    against a resident graph; p50/p99 latency and embeddings/s per rate, every
    result checked against the query's plain (fm_match) count."""
    import torch
    import forkmatch_gb300 as fm
    from forkmatch_gb300 import synth as S
    from forkmatch_gb300 import workloads as W
    if world > 1:
        raise SystemExit("--workload serving runs on one GPU")
    torch.cuda.set_device(local)
    scale = args.serving_scale
    m = W.SERVING["m"] >> (W.SERVING["scale"] - scale)
    t = time.time()
    G = W.serving_graph(scale, m)
    src, dst, lab = G.directed()
    gen_s = time.time() - t
    ctx = fm.Context(prealloc_bytes=args.pool_gb * GB, soln_prealloc_bytes=24 * GB, output_prealloc_bytes=8 * GB,
                     bank_rows=1 << 16, device=local)
    t = time.time()
    g = fm.Graph.from_edges(ctx, G.V, G.n_elabels + 1, src, dst, lab)
    load_s = time.time() - t
    del src, dst, lab
    t = time.time()
    A = S.BigAdjacency(G)
    adj_s = time.time() - t

    # screening on the device: a 1/4096 then 1/256 root sample, then the full
    # plain count, which is the reference result of every request
    rng = np.random.default_rng(20261205)
    V = G.V
    queries, alone, alone_ms, texts = [], [], [], []
    tried = 0
    t = time.time()
    while len(queries) < args.serving_queries and tried < 40 * args.serving_queries:
        tried += 1
        k = int(rng.integers(4, 13))
        qq = S.query_walk_big(A, k, rng)
        if qq is None:
            continue
        text = qq.to_g_text()
        q = fm.Query.from_text(text)
        r = fm.match(ctx, g, q, mode=fm.MODE_COUNT, work_limit=1 << 25, allow_limit=True)
        if r.status != fm.FM_OK or r.device_ms > args.serving_max_ms:
            continue
        queries.append(q)
        texts.append(text)
        alone.append(r.count)
        alone_ms.append(r.device_ms)
    screen_s = time.time() - t
    if not queries:
        raise SystemExit("no candidate query passed the screen (work limit 2^25, %g ms)" % args.serving_max_ms)
    sizes = [qu.q for qu in queries]

    srv = fm.Server(ctx, g, slots=args.slots, max_batch=args.max_batch)
    sweep = []
    sampler = ClockSampler(local)
    try:
        for rate in [float(x) for x in args.rates.split(",")]:
            n = int(min(args.serving_requests, max(50, rate * args.serving_seconds)))
            arr = np.cumsum(rng.exponential(1.0 / rate, size=n))
            pick = rng.integers(0, len(queries), size=n)
            tickets = []
            t0 = time.perf_counter()
            for i in range(n):
                target = t0 + arr[i]
                while True:
                    now = time.perf_counter()
                    if now >= target:
                        break
                    if target - now > 0.0005:
                        time.sleep(target - now - 0.0003)
                tickets.append(srv.submit(queries[pick[i]]))
            res = [srv.poll(tk) for tk in tickets]
            wall = time.perf_counter() - t0
            for tk in tickets:
                srv.release(tk)
            lat = np.array([r.latency_ms for r in res])
            emb = sum(r.count for r in res)
            sweep.append({"offered_qps": rate, "requests": n, "achieved_qps": n / wall,
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                          "mean_queue_ms": float(np.mean([r.queue_ms for r in res])),
                          "embeddings_per_s": emb / wall, "embeddings": emb,
                          "batched_requests": int(sum(1 for r in res if r.batch > 1)),
                          "bitexact": all(r.status == fm.FM_OK and r.count == alone[p] for r, p in zip(res, pick)),
                          "wall_s": wall})
        st = srv.stats()
    finally:
        clocks = sampler.stop()
        srv.close()
    top = sweep[-1]
    line = {"metric": METRIC, "value": top["embeddings_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": len(sweep), "warmup": 0, "ms_per_step": 1000 * top["wall_s"], "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generators)",
            "config": {"workload": "serving", "graph": "R-MAT(0.57,0.19,0.19,0.05) 2^%d vertices, %dM undirected "
                       "edges, 64 edge labels, 8 vertex labels uniform" % (scale, m // 1000000),
                       "queries": len(queries), "query_vertices": "%d-%d" % (min(sizes), max(sizes)),
                       "screening": "walk-induced subgraphs; kept when the plain count finishes within a work "
                                    "limit of 2^25 embeddings / partial matches and %g ms" % args.serving_max_ms,
                       "pool_gb": args.pool_gb, "slots": args.slots, "max_batch": args.max_batch,
                       "arrivals": "Poisson, %g s or %d requests per rate" % (args.serving_seconds,
                                                                             args.serving_requests)},
            "serving": sweep,
            "plain_alone": {"p50_device_ms": float(np.percentile(alone_ms, 50)),
                            "p99_device_ms": float(np.percentile(alone_ms, 99)),
                            "mean_count": float(np.mean(alone))},
            "pool": {"bytes": st.pool_bytes, "peak_used": st.pool_peak_used, "batches": st.batches},
            "clocks": clocks,
            "setup_s": {"generate": gen_s, "load": load_s, "adjacency": adj_s, "screen": screen_s,
                        "candidates": tried}}
    print(json.dumps(line), flush=True)
    g.close()
    ctx.close()
    return 0


def run_skew(args, rank, world, local):
    """Skewed low-selectivity stress: count-only stars, 4-cycles and 4-cliques
    on a Chung-Lu graph with hubs, every match bounded by a work limit; level
    buffers kept small so that hub chunks defer and drain.  Bit-exactness is
    checked on root samples the oracle finishes."""
    import torch
    import forkmatch_gb300 as fm
    from forkmatch_gb300 import synth as S
    from forkmatch_gb300 import workloads as W
    from oracle import oracle as O
    if world > 1:
        raise SystemExit("--workload skew runs on one GPU")
    torch.cuda.set_device(local)
    t = time.time()
    G = W.skew_graph()
    src, dst, lab = G.directed()
    gen_s = time.time() - t
    ctx = fm.Context(prealloc_bytes=8 * GB, soln_prealloc_bytes=4 * GB, output_prealloc_bytes=1 * GB,
                     bank_rows=1 << 20, device=local)
    g = fm.Graph.from_edges(ctx, G.V, G.n_elabels + 1, src, dst, lab)
    info = g.info()
    og = O.Graph.from_edges(G.V, G.n_elabels + 1, src, dst, lab)
    shapes = [("star5", S.query_star(5, [1, 1, 1, 1]), [1, 1, 1, 1]),
              ("star5_mixed", S.query_star(5, [1, 1, 2, 2]), [1, 1, 2, 2]),
              ("cycle4", S.query_cycle(4, [1, 1, 1, 1]), None), ("cycle4_mixed", S.query_cycle(4, [1, 2, 1, 2]), None),
              ("clique4", S.query_clique(4, [1]), None), ("clique4_mixed", S.query_clique(4, [1, 2]), None)]
    limit = args.skew_limit
    out = []
    tot_count = 0
    tot_ms = 0.0
    for name, qq, leaves in shapes:
        text = qq.to_g_text()
        q = fm.Query.from_text(text)
        fm.match(ctx, g, q, mode=fm.MODE_COUNT, roots=(0, 1024))   # warm-up
        r = fm.match(ctx, g, q, mode=fm.MODE_COUNT, work_limit=limit, allow_limit=True)
        row = {"query": name, "status": "complete" if r.status == fm.FM_OK else "work limit reached",
               "count": int(r.count), "device_ms": r.device_ms, "launches": int(r.launches),
               "embeddings_per_s": r.count / (r.device_ms / 1000.0) if r.device_ms > 0 else None}
        if leaves is not None:
            row["closed_form_count"] = W.star_count_closed_form(G, leaves)
        # bit-exact on root samples the oracle finishes (hub roots skipped)
        p = O.plan(text, enumerate_aut=0)
        checked = []
        for start in range(0, G.V, 4096):
            if len(checked) >= 3:
                break
            try:
                oc = O.match(og, p, roots=(start, start + 64), limit=1 << 24, scan_limit=1 << 28)[0]
            except O.OracleError:
                continue
            gc = fm.match(ctx, g, q, mode=fm.MODE_COUNT, roots=(start, start + 64)).count
            checked.append({"roots": [start, start + 64], "oracle": int(oc), "gpu": int(gc)})
        row["samples"] = checked
        row["samples_bitexact"] = bool(checked) and all(c["oracle"] == c["gpu"] for c in checked)
        out.append(row)
        tot_count += r.count
        tot_ms += r.device_ms
    line = {"metric": METRIC, "value": tot_count / (tot_ms / 1000.0), "unit": UNIT, "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": tot_ms, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "u64 counts", "data": "synthetic (seeded generators)",
            "config": {"workload": "skew", "graph": "Chung-Lu 2^21 vertices, exponent 2.1, degree cap 2^20, 32M "
                       "undirected edges, 1 vertex label, 2 edge labels", "max_list": info.max_list,
                       "work_limit": limit, "soln_prealloc_gb": 4, "mode": "count only"},
            "queries": out, "generate_s": gen_s}
    print(json.dumps(line), flush=True)
    g.close()
    ctx.close()
    return 0


def run_plain_small(args, rank, world, local):
    """The small plain configuration: Erdos-Renyi 1000 vertices / 2000 edges
    with 87 edge labels (the er1000_l87 graph of tests/golden/match_cases.json)
    and its 22 queries, one fm_match at a time, beside the per-query "Kernel
    Time" the reference's own GPU build printed for the same queries on a
    GB300 (tests/golden/ref_matches.json).  Device time per query: the median
    over the timed steps (CUDA events inside the library)."""
    import torch
    import forkmatch_gb300 as fm
    from tests.helpers import load_golden, make_graph
    torch.cuda.set_device(local)
    case = [c for c in load_golden("match_cases.json") if c["graph"] == "er1000_l87"][0]
    ref = {e["query"]: e for g in load_golden("ref_matches.json")["graphs"] if g["graph"] == "er1000_l87"
           for e in g["cases"]}
    ctx = fm.Context(prealloc_bytes=2 * GB, soln_prealloc_bytes=512 << 20, output_prealloc_bytes=512 << 20,
                     device=local)
    g = fm.Graph.from_text(ctx, make_graph(case["params"]).to_g_text())
    rows = []
    for e in case["cases"]:
        q = fm.Query.from_text(e["text"].encode())
        for _ in range(args.warmup):
            fm.match(ctx, g, q, mode=fm.MODE_TABLE)
        ms = []
        for _ in range(args.steps):
            r = fm.match(ctx, g, q, mode=fm.MODE_TABLE)
            ms.append(r.device_ms)
            assert r.count == e["count"]
        rr = ref.get(e["query"], {})
        rows.append({"query": e["query"], "count": e["count"], "device_ms": float(np.median(ms)),
                     "reference_kernel_ms": 1000 * rr["kernel_s"] if rr.get("kernel_s") else None,
                     "reference_count": rr.get("count")})
    ours = sum(r["device_ms"] for r in rows)
    theirs = sum(r["reference_kernel_ms"] for r in rows if r["reference_kernel_ms"])
    n_ref = sum(1 for r in rows if r["reference_kernel_ms"])
    line = {"metric": "matching time per query", "value": ours / len(rows), "unit": "ms", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "data": "synthetic (seeded)",
            "config": {"workload": "plain_small", "graph": "Erdos-Renyi 1000 vertices, 2000 edges, 87 edge labels",
                       "queries": len(rows)},
            "reference_sm103a_kernel_ms_per_query": theirs / n_ref if n_ref else None,
            "queries": rows}
    print(json.dumps(line), flush=True)
    g.close()
    ctx.close()
    return 0


def run_ingest(args, rank, world, local):
    """Ingest of the batched workload's graph as .g text (over 2 GiB): the
    text parsed on the device (fm_graph_load_file), parsed on the host into
    a binary cache (fm_graph_write_cache), and the cache loaded; every graph
    must equal the one built from the edge arrays."""
    import tempfile
    import torch
    import forkmatch_gb300 as fm
    from forkmatch_gb300 import workloads as W
    torch.cuda.set_device(local)
    G = W.batched_graph()
    src, dst, lab = G.directed()
    t = time.time()
    text = G.to_g_text()
    text_s = time.time() - t
    ctx = fm.Context(prealloc_bytes=2 * GB, soln_prealloc_bytes=512 << 20, output_prealloc_bytes=512 << 20,
                     device=local)
    ref = fm.Graph.from_edges(ctx, G.V, G.n_elabels + 1, src, dst, lab).info()
    fields = ("vertices", "label_slots", "edges", "segments", "long_segments", "max_list", "nbr_words")
    out = {}
    with tempfile.TemporaryDirectory() as td:
        tp, cp = os.path.join(td, "batched.g"), os.path.join(td, "batched.fmgb")
        with open(tp, "wb") as f:
            f.write(text)
        del text
        for name, fn in (("device_parse", lambda: fm.Graph.from_file(ctx, tp)),
                         ("host_parse_to_cache", lambda: fm.write_graph_cache(tp, cp)),
                         ("cache_load", lambda: fm.Graph.from_file(ctx, cp))):
            t = time.time()
            g = fn()
            el = time.time() - t
            row = {"seconds": el}
            if g is not None:
                inf = g.info()
                row["same_graph"] = all(getattr(inf, f) == getattr(ref, f) for f in fields)
                row["device_build_ms"] = inf.build_ms
                g.close()
            out[name] = row
        size = os.path.getsize(tp)
    line = {"metric": "ingest GB/s (text bytes / seconds)", "value": size / out["device_parse"]["seconds"] / 1e9,
            "unit": "GB/s", "n_gpus": 1, "higher_is_better": True, "data": "synthetic (seeded generators)",
            "config": {"workload": "ingest", "graph": "the batched workload's R-MAT 2^22 / 64M edges as .g text",
                       "text_bytes": size, "over_2GiB": size > (2 << 30), "text_generate_s": text_s},
            "paths": out}
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def verify_rows(ctx, g, queries, qinfo, edges, roots, sample=2048):
    """Size-independent check: sampled table rows are injective and every query
    e-line maps onto a data e-line with the same label."""
    import forkmatch_gb300 as fm
    src, dst, lab = edges
    key = (src.astype(np.uint64) << np.uint64(32)) | dst.astype(np.uint64)
    order = np.argsort(key)
    skey = key[order]
    slab = lab[order]
    rng = np.random.default_rng(0)
    for q, qi in zip(queries, qinfo):
        cnt, rows, r = fm.match_table(ctx, g, q, max_rows=1 << 16)
        if rows.shape[0] == 0:
            continue
        pick = rows[rng.integers(0, rows.shape[0], size=min(sample, rows.shape[0]))]
        col_of = {}
        for c in range(qi.q):
            col_of[qi.order[qi.q - 1 - c]] = c
        if any(len(set(rw)) != qi.q for rw in pick.tolist()):
            return False
        # query e-lines from the compiled plan: requirement (depth d, anc) with its label
        for d in range(1, qi.q):
            for i in range(qi.nreq[d]):
                anc = qi.order[d - qi.req_climb[d][i]]
                new = qi.order[d]
                a = pick[:, col_of[anc]].astype(np.uint64)
                b = pick[:, col_of[new]].astype(np.uint64)
                k = (a << np.uint64(32)) | b
                pos = np.searchsorted(skey, k)
                pos = np.minimum(pos, len(skey) - 1)
                if not np.all(skey[pos] == k):
                    return False
                # some copy of that e-line carries the required label
                okl = np.zeros(len(k), dtype=bool)
                p2 = pos.copy()
                while True:
                    m = (p2 < len(skey)) & (skey[np.minimum(p2, len(skey) - 1)] == k)
                    if not m.any():
                        break
                    okl |= m & (slab[np.minimum(p2, len(skey) - 1)] == qi.req_label[d][i])
                    p2 = p2 + 1
                if not okl.all():
                    return False
    return True


def cpu_baseline(wl, G, edges, name):
    """The CPU port timed on a bounded sample of the workload: whole queries
    (every CPU_EVERY-th), each over the full root range, all host threads."""
    from oracle import oracle as O
    src, dst, lab = edges
    og = O.Graph.from_edges(G.V, G.n_elabels + 1, src, dst, lab)
    threads = os.cpu_count() or 1
    sample = oracle_sample(wl, CPU_EVERY.get(name, 1))
    plans = [O.plan(wl["queries"][i]["text"].encode(), enumerate_aut=0) for i in sample]
    t0 = time.perf_counter()
    c = 0
    for i, p in zip(sample, plans):
        c += O.match(og, p, threads=threads, count_rule=is_count_only(wl["queries"][i]))[0]
    el = time.perf_counter() - t0
    model = cpu_model()
    return {"value": c / el, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": model,
            "sample": "%d of the %d queries (every %d-th), each over the full root range: %d embeddings in %.1f s "
                      "on %d threads of %s" % (len(sample), len(wl["queries"]), CPU_EVERY.get(name, 1), c, el,
                                               threads, model)}


def main():
    args = parse_args()
    rank, world, local = dist_info()
    if args.ncu_step:
        return run_ncu_step(args)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "batched":
        return run_batched(args, rank, world, local)
    if args.workload == "plain_at_scale":
        return run_ours(args, rank, world, local)
    if args.workload == "plain_small":
        return run_plain_small(args, rank, world, local)
    if args.workload == "serving":
        return run_serving(args, rank, world, local)
    if args.workload == "skew":
        return run_skew(args, rank, world, local)
    if args.workload == "ingest":
        return run_ingest(args, rank, world, local)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
