"""Record the reference's own GPU matcher output on the seeded match-case
graphs (run on a machine with a GPU; writes ref_matches.json).

The reference binary is oracle/_ref/ref_matcher: src/smsm.cu built with
SYMMETRY undefined behind oracle/ref_matcher_probe.cu (oracle/build.py).  That
build counts every embedding and writes every row in the reference's column
order (column i = vertex matched at depth q-1-i of the reference's order).

Only queries the reference can take without trapping or forking are sent:
    * the reference planner accepts them (connected, 2 <= q <= 16);
    * at most 3 back edges at every depth (isoLoop traps above that,
      src/smsm.cu:887-899);
    * every query edge label is a label of the data graph (1..EL);
    * the partial matches of all depths fit one memory bank of one block
      (at most 700 000 rows, below the bank's spill mark of 2^20 - 256*512,
      src/smsm.cu:446-454), so no child grid is launched.
Everything else is recorded as skipped with the reason.

For every query the probe's count (the reference's "Soln Size") and sorted
table are compared with the oracle's (validating the reference against the
oracle); the fixture keeps the reference's count, its "Kernel Time", the
SHA-256 of its sorted table and, for tables up to 4096 rows, the rows.

Usage: python tests/golden/make_ref_matches.py [out.json]
"""
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

from oracle import build as OB  # noqa: E402
from oracle import oracle as O  # noqa: E402

BANK_ROWS_LIMIT = 700_000
ROWS_KEPT = 4096


def sorted_rows(rows):
    rows = np.asarray(rows, dtype=np.uint32)
    return rows[np.lexsort(rows.T[::-1])] if rows.size else rows.reshape(0, rows.shape[1] if rows.ndim == 2 else 0)


def table_sha(rows):
    return hashlib.sha256(np.ascontiguousarray(sorted_rows(rows), dtype="<u4").tobytes()).hexdigest()


def screen(p, case, n_labels):
    if p.q < 2:
        return "single-vertex query (isoInit reads the depth-1 header)"
    for d in range(1, p.q):
        if p.nreq[d] > 3:
            return "%d back edges at depth %d (the reference traps above 3)" % (p.nreq[d], d)
        for i in range(p.nreq[d]):
            if not 1 <= p.req_label[d][i] <= n_labels:
                return "edge label %d outside the data graph's 1..%d" % (p.req_label[d][i], n_labels)
    if sum(case["partials"]) > BANK_ROWS_LIMIT:
        return "%d partial matches would fork child grids" % sum(case["partials"])
    return None


def run_probe(exe, qpath, gpath, q, timeout=180):
    r = subprocess.run([exe, qpath, gpath], capture_output=True, text=True, timeout=timeout)
    out = r.stdout
    res = {"rc": r.returncode}
    m = re.search(r"Soln Size: (\d+)", out)
    res["count"] = int(m.group(1)) if m else None
    m = re.search(r"Kernel Time: ([0-9.eE+-]+)s", out)
    res["kernel_s"] = float(m.group(1)) if m else None
    m = re.search(r"PROBE_ROWS (\d+)([ 0-9]*)", out)
    if m:
        words = np.array(m.group(2).split(), dtype=np.uint64).astype(np.uint32)
        res["rows"] = words.reshape(-1, q) if q else words
    else:
        res["rows"] = None
        res["tail"] = out[-2000:] + r.stderr[-2000:]
    return res


def main():
    from make_golden import make_graph
    out_path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_matches.json")
    OB.build_oracle()
    exe = OB.build_ref_matcher()
    if exe is None:
        raise SystemExit("the reference sources are not available (neither the checkout nor oracle/_ref/src)")
    cases_in = json.load(open(os.path.join(HERE, "match_cases.json")))
    result = []
    with tempfile.TemporaryDirectory() as td:
        for gc in cases_in:
            G = make_graph(gc["params"])
            text = G.to_g_text()
            assert hashlib.sha256(text).hexdigest() == gc["sha256"], gc["graph"]
            gpath = os.path.join(td, gc["graph"] + ".g")
            with open(gpath, "wb") as f:
                f.write(text)
            og = O.Graph.parse(text)
            entries = []
            for case in gc["cases"]:
                qtext = case["text"].encode()
                p = O.plan(qtext, enumerate_aut=0)
                why = screen(p, case, gc["params"]["n_elabels"])
                e = {"query": case["query"], "q": p.q}
                if why:
                    e["skipped"] = why
                    entries.append(e)
                    print(gc["graph"], case["query"], "skipped:", why, flush=True)
                    continue
                qpath = os.path.join(td, "q.g")
                with open(qpath, "wb") as f:
                    f.write(qtext)
                r = run_probe(exe, qpath, gpath, p.q)
                oc, orows, _ = O.match(og, p, table=True, table_cap=max(1, case["count"]))
                e.update({"rc": r["rc"], "count": r["count"], "kernel_s": r["kernel_s"], "oracle_count": int(oc)})
                if r["rows"] is not None:
                    e["rows_words"] = int(r["rows"].size)
                    e["table_sha256"] = table_sha(r["rows"])
                    e["oracle_table_sha256"] = table_sha(orows)
                    if r["rows"].shape[0] <= ROWS_KEPT:
                        e["rows"] = sorted_rows(r["rows"]).tolist()
                else:
                    e["tail"] = r.get("tail")
                e["agrees_with_oracle"] = bool(r["count"] == oc and e.get("table_sha256") == e.get("oracle_table_sha256"))
                entries.append(e)
                print(gc["graph"], case["query"], "count", r["count"], "oracle", oc, "kernel", r["kernel_s"],
                      "agree", e["agrees_with_oracle"], flush=True)
            result.append({"graph": gc["graph"], "params": gc["params"], "sha256": gc["sha256"], "cases": entries})
    with open(out_path, "w") as f:
        json.dump({"reference_build": "src/smsm.cu without SYMMETRY, nvcc -rdc=true sm_103a (oracle/build.py)",
                   "graphs": result}, f, indent=0)
    ran = [e for g in result for e in g["cases"] if "count" in e]
    print("ran", len(ran), "agree", sum(e["agrees_with_oracle"] for e in ran),
          "skipped", sum(1 for g in result for e in g["cases"] if "skipped" in e))


if __name__ == "__main__":
    main()
