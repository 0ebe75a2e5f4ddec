"""Host-side arithmetic of bench.py that needs no GPU: the algorithmic bytes
charged to a match (only what the kernels store or read: rows of stored
levels, record lookups, looked-up lists, table rows) and the DRAM traffic
figure scaled from the committed ncu summary, per kernel family."""
import types

import pytest

import bench


def _result(levels, count, pre_counted=0):
    """A stand-in for fm.Result: level[d] with lookups, list_words, produced."""
    lv = [types.SimpleNamespace(lookups=a, list_words=b, produced=c) for a, b, c in levels]
    return types.SimpleNamespace(level=lv, count=count, pre_counted=pre_counted)


def _info(q, nreq):
    return types.SimpleNamespace(q=q, nreq=nreq)


def test_table_match_charges_stored_levels_and_rows():
    # q = 4: depths 1, 2 store rows, depth 3 writes the table (4q bytes per row)
    r = _result([(0, 0, 0), (10, 40, 30), (60, 200, 50), (100, 300, 7)], count=7)
    qi = _info(4, [0, 1, 2, 2])
    want = (16 * 10 + 4 * 40 + 8 * 30) + (16 * 60 + 4 * 200 + 8 * 50) + (16 * 100 + 4 * 300) + 4 * 4 * 7
    assert bench.match_alg_bytes(r, qi, False) == want


def test_count_rule_last_depth_charges_its_lookups_only():
    # count only, last depth with one back edge: no list words, nothing stored
    r = _result([(0, 0, 0), (10, 40, 30), (30, 90, 80), (80, 5000, 123456)], count=123456)
    qi = _info(4, [0, 1, 1, 1])
    want = (16 * 10 + 4 * 40 + 8 * 30) + (16 * 30 + 4 * 90 + 8 * 80) + 16 * 80
    assert bench.match_alg_bytes(r, qi, True) == want


def test_pre_counted_depth_stores_nothing():
    # pre-count: depth q-2 = 2 counts its survivors, which are never stored
    r = _result([(0, 0, 0), (10, 40, 30), (30, 90, 80), (80, 5000, 123456)], count=123456, pre_counted=1)
    qi = _info(4, [0, 1, 1, 1])
    want = (16 * 10 + 4 * 40 + 8 * 30) + (16 * 30 + 4 * 90) + 16 * 80
    assert bench.match_alg_bytes(r, qi, True) == want


def test_count_only_last_depth_with_two_back_edges_reads_its_lists():
    # a count-only cycle: its last depth enumerates (two lists), but stores nothing
    r = _result([(0, 0, 0), (10, 40, 30), (60, 200, 50), (100, 300, 7)], count=7)
    qi = _info(4, [0, 1, 1, 2])
    want = (16 * 10 + 4 * 40 + 8 * 30) + (16 * 60 + 4 * 200 + 8 * 50) + (16 * 100 + 4 * 300)
    assert bench.match_alg_bytes(r, qi, True) == want


def test_batched_traffic_uses_both_kernel_families():
    ratios = {}
    with open(bench.os.path.join(bench.ROOT, "profiles", "k_bexpand_batched.md")) as f:
        for line in f:
            for key in ("traffic_bytes_per_algorithmic_byte", "traffic_bytes_per_algorithmic_byte_single"):
                if line.startswith(key + ":"):
                    ratios[key] = float(line.split(":")[1])
    assert len(ratios) == 2
    got = bench.batched_traffic(1_000_000_000, 3_000_000_000)
    want = 1e9 * ratios["traffic_bytes_per_algorithmic_byte"] + 3e9 * ratios["traffic_bytes_per_algorithmic_byte_single"]
    assert got == pytest.approx(want, rel=1e-9)
