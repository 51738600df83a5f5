// qd_common.cuh -- device building blocks of the QuIDS rule step:
// complex<double> magnitudes with the reference's rounding, unaligned byte
// access, the default object hasher and the 128-bit fixed-point accumulator
// used for the deterministic collision sum.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define QD_HD __host__ __device__ __forceinline__
#define QD_HD_CALL __host__ __device__ inline __noinline__  // a real call: one copy of the code
#define QD_D __device__ __forceinline__
#else
#define QD_HD inline
#define QD_HD_CALL inline
#define QD_D inline
#endif

namespace qd {

// ------------------------------------------------------------------ mag_t
// std::complex<double> as the reference computes it on x86-64 without FMA
// contraction (PROBA_TYPE double, src/quids.hpp:21-23, :78): every product and
// sum is rounded separately, so a child magnitude equals the reference's bit
// for bit.
struct mag_t {
    double re, im;
};

QD_HD double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
QD_HD double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
QD_HD double dsub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
QD_HD mag_t cmul(mag_t a, mag_t b) {
    return {dsub(dmul(a.re, b.re), dmul(a.im, b.im)), dadd(dmul(a.re, b.im), dmul(a.im, b.re))};
}
QD_HD mag_t cscale(mag_t a, double s) { return {dmul(a.re, s), dmul(a.im, s)}; }
QD_HD mag_t cneg(mag_t a) { return {-a.re, -a.im}; }
QD_HD mag_t cconj(mag_t a) { return {a.re, -a.im}; }
// std::norm(complex<double>) = re*re + im*im
QD_HD double cnorm(mag_t a) { return dadd(dmul(a.re, a.re), dmul(a.im, a.im)); }

// ------------------------------------------------------------ byte access
// Objects start at any byte offset (align_byte_length may be 0 or 1), and
// QCGD name sub-nodes sit at offset 4+4n of an object, misaligned for even n
// (src/rules/qcgd.hpp:85-94); these helpers never issue a misaligned access.
QD_HD uint16_t ld_u16(const char *p) {
    const unsigned char *q = (const unsigned char *)p;
    if (((uintptr_t)p & 1) == 0) return *(const uint16_t *)p;
    return (uint16_t)(q[0] | (q[1] << 8));
}
QD_HD void st_u16(char *p, uint16_t v) {
    if (((uintptr_t)p & 1) == 0) {
        *(uint16_t *)p = v;
        return;
    }
    p[0] = (char)(v & 0xff);
    p[1] = (char)(v >> 8);
}
QD_HD uint32_t ld_u32(const char *p) {
    if (((uintptr_t)p & 3) == 0) return *(const uint32_t *)p;
    const unsigned char *q = (const unsigned char *)p;
    return (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24);
}
QD_HD uint64_t ld_u64(const char *p) {
    uintptr_t a = (uintptr_t)p;
    if ((a & 7) == 0) return *(const uint64_t *)p;
    if ((a & 3) == 0) return (uint64_t)(*(const uint32_t *)p) | ((uint64_t)(*(const uint32_t *)(p + 4)) << 32);
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i) v = (v << 8) | (unsigned char)p[i];
    return v;
}
QD_HD void st_u64(char *p, uint64_t v) {
    uintptr_t a = (uintptr_t)p;
    if ((a & 7) == 0) {
        *(uint64_t *)p = v;
    } else if ((a & 3) == 0) {
        *(uint32_t *)p = (uint32_t)v;
        *(uint32_t *)(p + 4) = (uint32_t)(v >> 32);
    } else {
        for (int i = 0; i < 8; ++i) p[i] = (char)(v >> (8 * i));
    }
}
// copy n bytes; word copies when both ends share 8- or 4-byte alignment
QD_HD void copy_bytes(char *dst, const char *src, uint32_t n) {
    uintptr_t d = (uintptr_t)dst, s = (uintptr_t)src;
    uint32_t i = 0;
    if (((d ^ s) & 7) == 0) {
        for (; i < n && ((d + i) & 7); ++i) dst[i] = src[i];
        for (; i + 8 <= n; i += 8) *(uint64_t *)(dst + i) = *(const uint64_t *)(src + i);
    } else if (((d ^ s) & 3) == 0) {
        for (; i < n && ((d + i) & 3); ++i) dst[i] = src[i];
        for (; i + 4 <= n; i += 4) *(uint32_t *)(dst + i) = *(const uint32_t *)(src + i);
    }
    for (; i < n; ++i) dst[i] = src[i];
}

// --------------------------------------------------------- default hasher
// The reference's default hasher is std::hash<std::string_view>
// (src/quids.hpp:143-145); libstdc++ implements it as MurmurHash64A
// (Austin Appleby's published MurmurHash2, 64-bit variant) with seed
// 0xc70f6907.  Restated here; the tests pin it against std::hash.
constexpr uint64_t kMurmurMul = 0xc6a4a7935bd1e995ull;
constexpr uint64_t kStdHashSeed = 0xc70f6907ull;

QD_HD uint64_t murmur_shift_mix(uint64_t v) { return v ^ (v >> 47); }

// hash of `len` bytes at p, with byte `patch_pos` XOR-ed by `patch_xor`
// (patch_xor = 0 -> plain hash); lets a child that differs from its parent
// in one byte be hashed straight from the parent.
QD_HD uint64_t murmur64a_patched(const char *p, uint64_t len, uint64_t patch_pos, uint8_t patch_xor) {
    uint64_t h = kStdHashSeed ^ (len * kMurmurMul);
    uint64_t nblocks = len >> 3;
    for (uint64_t b = 0; b < nblocks; ++b) {
        uint64_t k = ld_u64(p + 8 * b);
        if ((patch_pos >> 3) == b) k ^= (uint64_t)patch_xor << (8 * (patch_pos & 7));
        k = murmur_shift_mix(k * kMurmurMul) * kMurmurMul;
        h ^= k;
        h *= kMurmurMul;
    }
    uint32_t tail = (uint32_t)(len & 7);
    if (tail) {
        const unsigned char *q = (const unsigned char *)p + 8 * nblocks;
        uint64_t k = 0;
        for (int i = (int)tail - 1; i >= 0; --i) k = (k << 8) | q[i];
        if ((patch_pos >> 3) == nblocks) k ^= (uint64_t)patch_xor << (8 * (patch_pos & 7));
        h ^= k;
        h *= kMurmurMul;
    }
    h = murmur_shift_mix(h) * kMurmurMul;
    return murmur_shift_mix(h);
}
QD_HD uint64_t murmur64a(const char *p, uint64_t len) { return murmur64a_patched(p, len, ~0ull, 0); }

// --------------------------------------------------- 128-bit fixed point
// Collision sums (src/quids.hpp:799-806) are accumulated exactly: each
// component is converted to a two's-complement 128-bit integer in units of
// 2^-F and added with 64-bit atomics (low word, then high word plus carry).
// Integer addition is associative, so the group sum is the same whatever the
// order of the children -- deterministic without a sort.
struct fix128 {
    uint64_t lo, hi;
};

QD_HD double pow2(int k) {
    // 2^k for -1022 <= k <= 1023
    uint64_t bits = (uint64_t)(k + 1023) << 52;
    double d;
    memcpy(&d, &bits, 8);
    return d;
}

QD_HD fix128 to_fix(double x, int F) {
    uint64_t bits;
    memcpy(&bits, &x, 8);
    fix128 r{0, 0};
    int ex = (int)((bits >> 52) & 0x7ff);
    if (ex == 0) return r;  // zero or subnormal (< 2^-1022): below any representable unit
    uint64_t man = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    int s = ex - 1075 + F;  // x = man * 2^(ex-1075); value = man * 2^s
    if (s >= 128) {
        r.lo = 0;
        r.hi = 0;  // out of range; scale guarantees this never happens
    } else if (s >= 64) {
        r.hi = man << (s - 64);
    } else if (s > 0) {
        r.lo = man << s;
        r.hi = man >> (64 - s);
    } else if (s == 0) {
        r.lo = man;
    } else if (s > -64) {
        r.lo = man >> (-s);
    }
    if (bits >> 63) {  // negate
        r.lo = ~r.lo + 1;
        r.hi = ~r.hi + (r.lo == 0 ? 1 : 0);
    }
    return r;
}

QD_HD int clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

QD_HD double u64_to_double_rn(uint64_t v) {
#ifdef __CUDA_ARCH__
    return __ull2double_rn(v);
#else
    return (double)v;
#endif
}

QD_HD fix128 fix_add(fix128 a, fix128 b) {
    fix128 r;
    r.lo = a.lo + b.lo;
    r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ull : 0ull);
    return r;
}

// correctly rounded (hi:lo) * 2^-F
QD_HD double from_fix(fix128 v, int F) {
    bool neg = (v.hi >> 63) != 0;
    if (neg) {
        v.lo = ~v.lo + 1;
        v.hi = ~v.hi + (v.lo == 0 ? 1 : 0);
    }
    if (v.hi == 0 && v.lo == 0) return 0.0;
    int lz = v.hi ? clz64(v.hi) : 64 + clz64(v.lo);
    // shift so the leading one is bit 127, keep the top 64 bits + sticky
    uint64_t top, rest;
    if (lz >= 64) {
        top = v.lo << (lz - 64);
        rest = 0;
    } else if (lz == 0) {
        top = v.hi;
        rest = v.lo;
    } else {
        top = (v.hi << lz) | (v.lo >> (64 - lz));
        rest = v.lo << lz;
    }
    if (rest) top |= 1;
    double d = u64_to_double_rn(top);  // value = top * 2^(64 - lz)
    int k = 64 - lz - F;
    while (k < -1022) {
        d *= pow2(-1022);
        k += 1022;
    }
    while (k > 1023) {
        d *= pow2(1023);
        k -= 1023;
    }
    d *= pow2(k);
    return neg ? -d : d;
}

// F such that |sum| < 2^125 * 2^-F for n terms of magnitude <= maxabs
QD_HD int fix_scale(double maxabs, uint64_t n) {
    if (!(maxabs > 0)) return 0;
    uint64_t bits;
    memcpy(&bits, &maxabs, 8);
    int e = (int)((bits >> 52) & 0x7ff) - 1022;  // maxabs < 2^e
    const int ln = n <= 1 ? 0 : 64 - clz64(n - 1);  // n <= 2^ln
    return 124 - e - ln;
}

}  // namespace qd
