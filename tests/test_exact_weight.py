"""sum_minus_scaled (csrc/exact_weight.cuh) must equal the FP64 expression
ldexp(fl(a + b) - c, St) bit for bit. The header compiles for the host; this
CPU test builds a small driver with g++ and checks millions of cases: random
pivot-like operands, exact ties of the rounding, carries into the next binade,
b far below a's last place, c on both sides of fl(a + b)."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300", "csrc")

DRIVER = r"""
#include "exact_weight.cuh"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
using namespace pbe_gb300;

static uint64_t bits(double v) { uint64_t u; std::memcpy(&u, &v, 8); return u; }
static double from(uint64_t u) { double v; std::memcpy(&v, &u, 8); return v; }
static long bad = 0, total = 0;

static void check(double a, double b, double c, int St) {
    if (!(b <= a) || !(a > 0) || !(b > 0) || !(c > 0)) return;
    double s = a + b;
    int es = std::ilogb(s), ec = std::ilogb(c);
    if (std::abs(es - ec) > kMaxExpGap) return;
    double want = std::ldexp(s - c, St);
    if (want != 0.0 && !std::isnormal(want)) return;
    double got = sum_minus_scaled(a, b, c, St);
    ++total;
    if (bits(got) != bits(want)) {
        if (bad < 10) std::printf("MISMATCH a=%a b=%a c=%a St=%d got=%a want=%a\n", a, b, c, St, got, want);
        ++bad;
    }
}

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    // random pivot-like operands on grids with ratio 2^(1/q)
    for (int it = 0; it < 2000000; ++it) {
        double a = std::ldexp(1.0 + U(rng), (int)(rng() % 200) - 100);
        int gap = (int)(rng() % 70);
        double b = std::ldexp(1.0 + U(rng), std::ilogb(a) - gap);
        if (b > a) b = a;
        double s = a + b;
        double c;
        switch (rng() % 5) {
        case 0: c = a; break;
        case 1: c = s; break;
        case 2: c = std::nextafter(s, 0.0); break;
        case 3: c = s * (1.0 - 0.01 * U(rng)); break;
        default: c = std::nextafter(s, 1e300); break;
        }
        int St = -std::ilogb(c) + (int)(rng() % 7) - 3;
        check(a, b, c, St);
    }
    // exact ties: b = half an ulp of a (and odd/even a), plus sticky variants
    for (int it = 0; it < 200000; ++it) {
        double a = std::ldexp(1.0 + U(rng), (int)(rng() % 40) - 20);
        uint64_t ua = bits(a);
        if (rng() & 1) ua |= 1; else ua &= ~1ull;
        a = from(ua);
        int k = 1 + (int)(rng() % 60);                   // b = (odd) * 2^-k ulp
        double ulp = std::nextafter(a, 1e300) - a;
        double b = std::ldexp(ulp, -1);                  // exact half ulp
        if (rng() & 1) b = b + std::ldexp(ulp, -1 - k);  // just above half
        if (rng() % 3 == 0) b = b - std::ldexp(ulp, -1 - k);
        check(a, b, a, -std::ilogb(a));
        check(a, b, a + b, -std::ilogb(a));
    }
    // carries: a just below a power of two
    for (int it = 0; it < 200000; ++it) {
        int e = (int)(rng() % 60) - 30;
        double a = std::nextafter(std::ldexp(1.0, e), 0.0);
        for (int s = 0; s < (int)(rng() % 8); ++s) a = std::nextafter(a, 0.0);
        double b = std::ldexp(U(rng), e - (int)(rng() % 56));
        if (b <= 0) continue;
        check(a, b, std::ldexp(1.0, e), -e);
        check(a, b, a, -e);
    }
    // geometric grids as used by the library: x_j + x_{j+d} against x_lo
    for (int q : {1, 3, 16, 128, 512}) {
        const int n = 3000;
        std::vector<double> x(n);
        for (int i = 0; i < n; ++i) x[i] = 1e-21 * std::pow(2.0, i / (double)q);
        for (int it = 0; it < 200000; ++it) {
            int j = (int)(rng() % n), d = (int)(rng() % (n - j));
            double v = x[j] + x[j + d];
            int lo = (int)(std::upper_bound(x.begin(), x.end(), v) - x.begin()) - 1;
            if (lo < 0 || lo >= n - 1) continue;
            for (int dl = -1; dl <= 0; ++dl)
                if (lo + dl >= j + d) check(x[j + d], x[j], x[lo + dl], -std::ilogb(x[lo]));
        }
    }
    std::printf("%ld %ld\n", total, bad);
    return bad != 0;
}
"""


def test_sum_minus_scaled_is_bit_exact():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "drv.cpp")
        exe = os.path.join(d, "drv")
        with open(src, "w") as f:
            f.write(DRIVER.replace("#include <random>", "#include <random>\n#include <vector>\n#include <algorithm>"))
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC, src, "-o", exe],
                       check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
        last = out.stdout.strip().splitlines()[-1].split()
        total, bad = int(last[0]), int(last[1])
        assert total > 2_000_000, out.stdout
        assert bad == 0, out.stdout
