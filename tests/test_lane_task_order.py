"""The launch order of the lane tasks (pbe_internal.cuh: lane_full_tasks,
lane_last_rank for the forward pair kernel; vjp_lane_full_tasks,
vjp_lane_last_rank for the VJP): a host driver built with nvcc rebuilds the
tables the prep kernels write and checks that each is a permutation of the
(block, chunk) tasks, with the full chunks first and the last chunks in
non-increasing length. No GPU needed."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300", "csrc")

DRIVER = r"""
#include "pbe_internal.cuh"
#include <cstdio>
#include <set>
#include <utility>
#include <vector>
using namespace pbe_gb300;

static int fails = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL n=%d line %d\n", n, __LINE__); ++fails; return; } } while (0)

static void forward(int n)
{
    const int C = lane_chunk_len(n);
    const int T = static_cast<int>(lane_tasks(n, C)), full = lane_full_tasks(n, C);
    std::vector<std::pair<int, int>> tab(T, {-1, -1});
    for (int i = 0; i < full; ++i) {                   // as agg_prep_kernel
        int r = i, c = 0;
        while (r >= lane_chunk_blocks(n, c + 1, C)) { r -= lane_chunk_blocks(n, c + 1, C); ++c; }
        tab[i] = {r, c};
    }
    for (int t = 0; t < lane_blocks(n); ++t) {
        const int k = full + lane_last_rank(n, t, C);
        CHECK(k >= full && k < T && tab[k].first < 0);
        tab[k] = {t, lane_block_chunks(n, t, C) - 1};
    }
    std::set<std::pair<int, int>> want, got(tab.begin(), tab.end());
    for (int c = 0; lane_chunk_blocks(n, c, C) > 0; ++c)
        for (int t = 0; t < lane_chunk_blocks(n, c, C); ++t) want.insert({t, c});
    CHECK(got == want && static_cast<int>(want.size()) == T);
    for (int i = 0; i < full; ++i) CHECK(tab[i].second < lane_block_chunks(n, tab[i].first, C) - 1);
    for (int k = full + 1; k < T; ++k) {
        const int a = lane_last_chunk_len(n, tab[k - 1].first, C), b = lane_last_chunk_len(n, tab[k].first, C);
        CHECK((a > 0 ? a : 0) >= (b > 0 ? b : 0));
    }
}

static void vjp(int n)
{
    const int C = vjp_lane_chunk(n);
    const int T = static_cast<int>(vjp_lane_tasks(n, C)), full = vjp_lane_full_tasks(n, C);
    const int nvb = vjp_lane_chunk_blocks(n, 0, C);
    std::vector<std::pair<int, int>> tab(T, {-1, -1});
    for (int i = 0; i < full; ++i) {                   // as vjp_prep_kernel
        int r = i, c = 0;
        while (r >= vjp_lane_chunk_blocks(n, c + 1, C)) { r -= vjp_lane_chunk_blocks(n, c + 1, C); ++c; }
        tab[i] = {r, c};
    }
    for (int b = 0; b < nvb; ++b) {
        const int k = full + vjp_lane_last_rank(n, b, C);
        CHECK(k >= full && k < T && tab[k].first < 0);
        tab[k] = {b, (n - 1 - kLaneBins * b + C - 1) / C - 1};
    }
    std::set<std::pair<int, int>> want, got(tab.begin(), tab.end());
    for (int c = 0; vjp_lane_chunk_blocks(n, c, C) > 0; ++c)
        for (int b = 0; b < vjp_lane_chunk_blocks(n, c, C); ++b) want.insert({b, c});
    CHECK(got == want && static_cast<int>(want.size()) == T);
    auto len = [&](int b, int c) {
        const int dA = 1 + c * C, dB = dA + C < n - kLaneBins * b ? dA + C : n - kLaneBins * b;
        return dB - dA;
    };
    for (int i = 0; i < full; ++i) CHECK(len(tab[i].first, tab[i].second) == C);
    for (int k = full + 1; k < T; ++k)
        CHECK(len(tab[k - 1].first, tab[k - 1].second) >= len(tab[k].first, tab[k].second));
}

int main()
{
    int count = 0;
    for (int n = 1; n <= 2100; ++n) { forward(n); if (n >= 2) vjp(n); ++count; }
    for (int n : {3840, 4500, 8191, 8192, 8193, 12000, 16384, 20000, 32768}) { forward(n); vjp(n); ++count; }
    std::printf("%d %d\n", count, fails);
    return fails != 0;
}
"""


def test_lane_task_tables_are_sorted_permutations():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "order.cu")
        exe = os.path.join(d, "order")
        with open(src, "w") as f:
            f.write(DRIVER)
        subprocess.run([nvcc, "-std=c++17", "-O1", "-I" + CSRC, "-I" + os.path.join(ROOT, "include"),
                        src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout[-2000:]
        count, fails = map(int, out.stdout.strip().splitlines()[-1].split())
        assert fails == 0 and count > 2100
