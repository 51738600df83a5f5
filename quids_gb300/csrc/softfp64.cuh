// softfp64.cuh -- IEEE-754 binary64 multiply and add, rounded to nearest
// even, computed with integer instructions.
//
// GB300 issues FP64 arithmetic at about one operation per clock per SM, a
// small fraction of its integer rate (the FP32/INT32 lanes), and the rule
// step's complex magnitude products must be rounded exactly as the reference
// rounds them (every product and sum separately, no contraction).  These
// routines give the same bits as the hardware's __dmul_rn / __dadd_rn from
// integer multiplies, shifts and adds, written from the IEEE-754 definition
// of round-to-nearest-even (a 106-bit product or an aligned sum with guard
// bits and a sticky bit, then one rounding).
//
// Only finite operands and results in the normal range take the integer
// path.  Zeros, subnormals, infinities, NaNs and results that overflow or
// underflow the normal range are handed to the hardware instruction, which
// keeps those cases exact by construction.  tests/test_softfp64.py compares
// both routines with the host's IEEE arithmetic on hundreds of millions of
// operands, including exact ties, cancellations and every exponent gap.
#pragma once
#include <cstdint>
#include <cstring>

#if !defined(QD_HD)
#if defined(__CUDACC__)
#define QD_HD __host__ __device__ __forceinline__
#else
#define QD_HD inline
#endif
#endif

namespace qd::softfp {

constexpr uint64_t kSign = 1ull << 63;
constexpr uint64_t kMant = (1ull << 52) - 1;
constexpr uint64_t kHidden = 1ull << 52;

QD_HD uint64_t to_bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}
QD_HD double from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}
QD_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
QD_HD int clz(uint64_t v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
QD_HD double hw_mul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;  // no contraction on the host either
    return r;
#endif
}
QD_HD double hw_add(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    volatile double r = a + b;
    return r;
#endif
}

// a * b.  With both significands as 1.f * 2^63 in 64 bits, their product is
// (1.fa * 1.fb) * 2^126: its top 64 bits hold the leading one at bit 63 (a
// product in [2, 4)) or bit 62 (in [1, 2)); 53 bits are kept, the next bit
// is the rounding bit and every bit below it feeds the sticky bit.
QD_HD double mul(double x, double y) {
    const uint64_t a = to_bits(x), b = to_bits(y);
    const uint32_t ea = (uint32_t)(a >> 52) & 0x7ff, eb = (uint32_t)(b >> 52) & 0x7ff;
    if (ea - 1u >= 0x7feu || eb - 1u >= 0x7feu) return hw_mul(x, y);  // zero, subnormal, inf, nan
    const uint64_t ma = (a << 11) | kSign, mb = (b << 11) | kSign;
    uint64_t hi = mulhi64(ma, mb);
    uint64_t lo = ma * mb;
    int e = (int)ea + (int)eb - 1023;
    if (hi >> 63) {
        ++e;
    } else {
        hi = (hi << 1) | (lo >> 63);
        lo <<= 1;
    }
    uint64_t keep = hi >> 11;            // 53 bits, leading one at bit 52
    const uint64_t r = hi & 0x7ff;       // rounding bit 0x400, then 10 more bits
    const bool up = r > 0x400 || (r == 0x400 && (lo != 0 || (keep & 1)));
    keep += up ? 1 : 0;
    if (keep >> 53) {  // rounded up to 2.0
        keep >>= 1;
        ++e;
    }
    if (e <= 0 || e >= 0x7ff) return hw_mul(x, y);  // underflow or overflow
    return from_bits(((a ^ b) & kSign) | ((uint64_t)e << 52) | (keep & kMant));
}

// a + b.  The operand of larger magnitude first; significands carry 10
// guard bits (leading one at bit 62); the smaller one is shifted right with
// every bit shifted out OR-ed into its lowest bit (a sticky bit that keeps
// the result odd, so a discarded tail can never look like an exact tie).
// Only a difference of exponents of 0 or 1 can cancel more than one leading
// bit, and then no bit was shifted out, so the renormalised result is exact
// before rounding.
QD_HD double add(double x, double y) {
    uint64_t a = to_bits(x), b = to_bits(y);
    uint32_t ea = (uint32_t)(a >> 52) & 0x7ff, eb = (uint32_t)(b >> 52) & 0x7ff;
    if (ea - 1u >= 0x7feu || eb - 1u >= 0x7feu) return hw_add(x, y);
    if ((a & ~kSign) < (b & ~kSign)) {
        const uint64_t t = a;
        a = b;
        b = t;
        const uint32_t u = ea;
        ea = eb;
        eb = u;
    }
    const uint64_t ma = ((a & kMant) | kHidden) << 10;
    uint64_t mb = ((b & kMant) | kHidden) << 10;
    const uint32_t d = ea - eb;
    if (d > 62) {
        mb = 1;
    } else if (d) {
        const uint64_t lost = mb << (64 - d);
        mb = (mb >> d) | (lost != 0 ? 1ull : 0ull);
    }
    int e = (int)ea;
    uint64_t m;
    if (((a ^ b) & kSign) == 0) {
        m = ma + mb;
        if (m >> 63) {
            m = (m >> 1) | (m & 1);
            ++e;
        }
    } else {
        m = ma - mb;
        if (m == 0) return 0.0;  // exact cancellation: +0 when rounding to nearest
        const int s = clz(m) - 1;
        m <<= s;
        e -= s;
    }
    uint64_t keep = m >> 10;
    const uint64_t r = m & 0x3ff;  // rounding bit 0x200
    keep += (r > 0x200 || (r == 0x200 && (keep & 1))) ? 1 : 0;
    if (keep >> 53) {
        keep >>= 1;
        ++e;
    }
    if (e <= 0 || e >= 0x7ff) return hw_add(x, y);
    return from_bits((a & kSign) | ((uint64_t)e << 52) | (keep & kMant));
}

QD_HD double sub(double x, double y) { return add(x, from_bits(to_bits(y) ^ kSign)); }

}  // namespace qd::softfp
