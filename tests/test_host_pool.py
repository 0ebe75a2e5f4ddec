"""The server's lease allocator (forkmatch_gb300/csrc/fm_pool.h, host only)
against a unit-by-unit model: random leases and releases never overlap, the
free byte count and the largest free range are exact, and releasing
everything coalesces the pool back into one range."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include "fm_pool.h"

int main() {
    const uint64_t U = 64, N = 4096;            // units of 64 bytes, 4096 units
    fm::PoolAlloc pool;
    pool.init(U * N);
    std::vector<int> owner(N, -1);
    struct Lease { uint64_t off, bytes; };
    std::vector<Lease> live;
    std::mt19937_64 rng(7);
    for (int step = 0; step < 200000; step++) {
        if (live.empty() || rng() % 3) {
            const uint64_t bytes = U * (1 + rng() % 96);
            uint64_t off = 0;
            // the model: is there a free run of that many units?
            uint64_t run = 0, best = 0;
            for (uint64_t u = 0; u < N; u++) { run = owner[u] < 0 ? run + 1 : 0; if (run > best) best = run; }
            const bool ok = pool.alloc(bytes, off);
            if (ok != (best * U >= bytes)) { std::printf("fit mismatch at step %d\n", step); return 1; }
            if (pool.largest() > U * N) return 2;
            if (!ok) continue;
            if (off % U) return 3;
            for (uint64_t u = off / U; u < (off + bytes) / U; u++) {
                if (owner[u] >= 0) { std::printf("overlap at step %d\n", step); return 4; }
                owner[u] = (int)live.size();
            }
            live.push_back({off, bytes});
        } else {
            const size_t i = rng() % live.size();
            const Lease l = live[i];
            pool.release(l.off, l.bytes);
            for (uint64_t u = l.off / U; u < (l.off + l.bytes) / U; u++) owner[u] = -1;
            live[i] = live.back();
            live.pop_back();
            for (uint64_t u = 0; u < N; u++)
                if (owner[u] == (int)live.size()) owner[u] = (int)i;
        }
        uint64_t freeu = 0, run = 0, best = 0;
        for (uint64_t u = 0; u < N; u++) {
            if (owner[u] < 0) { freeu++; run++; } else run = 0;
            if (run > best) best = run;
        }
        if (pool.free_bytes() != freeu * U || pool.largest() != best * U) {
            std::printf("accounting mismatch at step %d\n", step);
            return 5;
        }
    }
    for (const auto& l : live) pool.release(l.off, l.bytes);
    if (pool.free_ranges() != 1 || pool.free_bytes() != U * N || pool.largest() != U * N) return 6;
    std::printf("ok peak %llu\n", (unsigned long long)pool.peak());
    return 0;
}
"""


def test_pool_allocator_against_a_model(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "pool_check.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "pool_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "forkmatch_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
