// =============================================================================
// exact_weight.cuh -- the fixed-pivot weight numerator fl(x_j + x_k) - x_lo,
// computed bit-exactly with integer instructions.
//
// On GB300 the FP64 pipe runs at 2 operations/clk/SM while the integer pipe is
// ~60x wider and idle in the pair loop. The reference forms the numerator with
// two FP64 additions (src/aggregation_kernels.cuh:190, :198); this function
// returns the identical IEEE-754 value -- round-to-nearest-even sum, exact
// difference -- times 2^St, without touching the FP64 pipe.
//
// Preconditions (the geometric path guarantees them: pivots are positive
// normal doubles, ratio between neighbours <= 2^kMaxExpGap / 2): a, b, c
// positive normal doubles; b <= a; the exponents of fl(a + b) and c differ by
// at most kMaxExpGap; the result times 2^St is a normal double or zero. The
// difference is rounded to nearest even like FP64 when it needs more than 53
// bits (only possible when fl(a + b) and c are more than a factor 2 apart).
// Compiles for the host as well, where tests compare it with FP64 arithmetic.
// =============================================================================
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define PBE_HD __host__ __device__ __forceinline__
#else
#define PBE_HD inline
#endif

namespace pbe_gb300 {

constexpr int kMaxExpGap = 8;

PBE_HD uint64_t ew_bits(double v)
{
#if defined(__CUDA_ARCH__)
    return static_cast<uint64_t>(__double_as_longlong(v));
#else
    uint64_t u;
    __builtin_memcpy(&u, &v, sizeof(u));
    return u;
#endif
}

PBE_HD double ew_double(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(u));
#else
    double v;
    __builtin_memcpy(&v, &u, sizeof(v));
    return v;
#endif
}

PBE_HD int ew_clz64(uint64_t v)
{
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(v));
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

// The operands that stay fixed over runs of calls in the pair loops, decoded
// once: a (the larger addend) as its 63-bit fixed-point significand and
// biased exponent, c (the subtrahend) with the result's scale St.
struct EwOperandA {
    uint64_t A;    // significand with the hidden bit, shifted left by 10 guard bits
    int ea;        // biased exponent
};
struct EwOperandC {
    uint64_t mc;   // significand with the hidden bit
    int ec;        // biased exponent
    int St;
};
PBE_HD EwOperandA ew_operand_a(double a)
{
    constexpr uint64_t kM52 = (1ull << 52) - 1;
    constexpr uint64_t kH53 = 1ull << 52;
    const uint64_t ua = ew_bits(a);
    return EwOperandA{((ua & kM52) | kH53) << 10, static_cast<int>(ua >> 52)};
}
PBE_HD EwOperandC ew_operand_c(double c, int St)
{
    constexpr uint64_t kM52 = (1ull << 52) - 1;
    constexpr uint64_t kH53 = 1ull << 52;
    const uint64_t uc = ew_bits(c);
    return EwOperandC{(uc & kM52) | kH53, static_cast<int>(uc >> 52), St};
}

// b (the smaller addend) decoded: significand with the hidden bit, shifted
// left by 10 guard bits, and biased exponent.
struct EwOperandB {
    uint64_t bw;
    int eb;
};
PBE_HD EwOperandB ew_operand_b(double b)
{
    constexpr uint64_t kM52 = (1ull << 52) - 1;
    constexpr uint64_t kH53 = 1ull << 52;
    const uint64_t ub = ew_bits(b);
    return EwOperandB{((ub & kM52) | kH53) << 10, static_cast<int>(ub >> 52)};
}

// (fl(a + b) - c) * 2^St from the decoded operands.
PBE_HD double sum_minus_scaled_dec(const EwOperandA& pa, const EwOperandB& pb, const EwOperandC& pc)
{
    constexpr uint64_t kM52 = (1ull << 52) - 1;

    // ---- s = fl(a + b), round to nearest even --------------------------------
    // a and b as 63-bit fixed point with 10 guard bits below a's last place.
    const int d = pa.ea - pb.eb;                 // >= 0 because b <= a
    const uint64_t A = pa.A;
    uint64_t B;
    bool sticky;
    if (d >= 64) {
        B = 0;
        sticky = true;                           // b != 0 lies entirely below
    } else {
        const uint64_t bw = pb.bw;
        B = bw >> d;
        sticky = d > 0 && (bw << (64 - d)) != 0;
    }
    const uint64_t S = A + B;                    // < 2^64 since B <= A < 2^63
    const int carry = static_cast<int>(S >> 63); // sum reached the next binade
    const int rs = 10 + carry;
    int es = pa.ea + carry;
    uint64_t ms = S >> rs;                       // 53 significant bits
    const uint64_t rem = S & ((1ull << rs) - 1);
    const uint64_t half = 1ull << (rs - 1);
    const bool up = rem > half || (rem == half && (sticky || (ms & 1u)));
    ms += up ? 1u : 0u;
    if (ms >> 53) { ms >>= 1; ++es; }            // rounding carried into a new binade

    // ---- t = s - c exactly (integers on the smaller of the two exponents) -----
    const int ec = pc.ec;
    const int e0 = es < ec ? es : ec;
    const int64_t T = static_cast<int64_t>(ms << (es - e0)) - static_cast<int64_t>(pc.mc << (ec - e0));
    if (T == 0) return 0.0;
    const uint64_t sign = T < 0 ? (1ull << 63) : 0ull;
    uint64_t m = T < 0 ? static_cast<uint64_t>(-T) : static_cast<uint64_t>(T);
    const int p = 63 - ew_clz64(m);              // leading bit, < 53 + kMaxExpGap
    int E = e0 + p - 52 + pc.St;                 // biased exponent of the result
    if (p <= 52) {
        m <<= (52 - p);
    } else {                                     // more than 53 bits: round to nearest even
        const int sh = p - 52;
        const uint64_t r = m & ((1ull << sh) - 1), h = 1ull << (sh - 1);
        m >>= sh;
        if (r > h || (r == h && (m & 1u))) {
            ++m;
            if (m >> 53) { m >>= 1; ++E; }
        }
    }
    return ew_double(sign | (static_cast<uint64_t>(E) << 52) | (m & kM52));
}

// The same with a and c decoded (b varies from call to call).
PBE_HD double sum_minus_scaled_pre(const EwOperandA& pa, double b, const EwOperandC& pc)
{
    return sum_minus_scaled_dec(pa, ew_operand_b(b), pc);
}

// Returns (fl(a + b) - c) * 2^St.
PBE_HD double sum_minus_scaled(double a, double b, double c, int St)
{
    return sum_minus_scaled_dec(ew_operand_a(a), ew_operand_b(b), ew_operand_c(c, St));
}

} // namespace pbe_gb300
