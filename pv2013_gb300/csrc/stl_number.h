// Exact decimal -> double conversion for the device STL parser, host and
// device code alike (plain C++ when not compiled by nvcc, so that the CPU
// tests can compare it with strtod on millions of strings).
//
// Scope: the decimal forms Reader::readSTLASCII accepts through
// istream >> double (GeometryReader.cpp:33-117): [sign] digits [. digits]
// [e|E [sign] digits].  A value is w * 10^e10 with w the decimal significand.
// It is converted exactly when w has at most 19 significant digits (any
// further digits zero) and |e10| <= 60, which covers the files STL writers
// produce (%.17g of coordinates and of normals with components near 1e-17);
// otherwise the converter reports that it cannot decide and the caller
// parses the text with strtod.
//
// Method (integer arithmetic, correct rounding to nearest, ties to even):
//   e10 >= 0:  N = w * 5^e10 (exact: 128 bits for e10 <= 27, where
//              5^27 < 2^63, else 256 bits); value = N * 2^e10; N is rounded
//              to 53 bits.
//   e10 <  0:  k = -e10; q = floor(w * 2^s / 5^k), r the remainder, s chosen
//              so that q has more than 55 bits (128-bit division by a 64-bit
//              5^k for k <= 27, else restoring division in 256 bits);
//              value = (q + r / 5^k) * 2^-(s + k); q is rounded to 53 bits
//              with r != 0 as the sticky bit.
// The 53-bit mantissa times a power of two is then exact in a double
// (the exponents stay inside the normal range for these inputs).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define LBM_HD __host__ __device__ __forceinline__
#else
#define LBM_HD inline
#endif

namespace lbm {
namespace stlnum {

struct U128 {
    uint64_t hi, lo;
};

LBM_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

LBM_HD U128 mul64(uint64_t a, uint64_t b) {
    // 64 x 64 -> 128 by 32-bit halves (same code on host and device)
    const uint64_t a0 = a & 0xffffffffull, a1 = a >> 32, b0 = b & 0xffffffffull, b1 = b >> 32;
    const uint64_t p00 = a0 * b0, p01 = a0 * b1, p10 = a1 * b0, p11 = a1 * b1;
    const uint64_t mid = (p00 >> 32) + (p01 & 0xffffffffull) + (p10 & 0xffffffffull);
    U128 r;
    r.lo = (p00 & 0xffffffffull) | (mid << 32);
    r.hi = p11 + (p01 >> 32) + (p10 >> 32) + (mid >> 32);
    return r;
}

LBM_HD uint64_t pow5(int k) {
    uint64_t p = 1;
    for (int i = 0; i < k; ++i) p *= 5u;
    return p;
}

// (hi:lo) / d with hi < d: quotient (64 bits) and remainder, by long division
LBM_HD uint64_t div128_small(uint64_t hi, uint64_t lo, uint64_t d, uint64_t* rem) {
    uint64_t r = hi, q = 0;
    for (int i = 63; i >= 0; --i) {
        const uint64_t top = r >> 63;
        r = (r << 1) | ((lo >> i) & 1u);
        q <<= 1;
        if (top || r >= d) { r -= d; q |= 1u; }
    }
    *rem = r;
    return q;
}

// m * 2^e as a double, m < 2^53 (exact for results in the normal range)
LBM_HD double scale2(uint64_t m, int e) {
    double v = (double)m;
    // multiply by powers of two in steps that keep every factor exact
    while (e > 0) { const int s = e > 60 ? 60 : e; v *= (double)(1ull << s); e -= s; }
    while (e < 0) { const int s = -e > 60 ? 60 : -e; v /= (double)(1ull << s); e += s; }
    return v;
}

LBM_HD U128 shr128(U128 n, int s) {
    U128 r;
    if (s == 0) return n;
    if (s < 64) { r.lo = (n.lo >> s) | (n.hi << (64 - s)); r.hi = n.hi >> s; }
    else { r.lo = n.hi >> (s - 64); r.hi = 0; }
    return r;
}
LBM_HD U128 shl128(U128 n, int s) {
    U128 r;
    if (s == 0) return n;
    if (s < 64) { r.hi = (n.hi << s) | (n.lo >> (64 - s)); r.lo = n.lo << s; }
    else { r.hi = n.lo << (s - 64); r.lo = 0; }
    return r;
}
LBM_HD int cmp128(U128 a, U128 b) {
    if (a.hi != b.hi) return a.hi < b.hi ? -1 : 1;
    if (a.lo != b.lo) return a.lo < b.lo ? -1 : 1;
    return 0;
}

// round the nonzero 128-bit integer n to 53 significant bits, to nearest
// with ties to even; sticky = nonzero value below n's last bit (then n is
// never exactly halfway).  Returns the mantissa m and sets *exp2 so that
// the rounded value is m * 2^exp2.
LBM_HD uint64_t round53(U128 n, bool sticky, int* exp2) {
    const int msb = n.hi ? 127 - clz64(n.hi) : 63 - clz64(n.lo);
    if (msb <= 52 && !sticky) {
        *exp2 = 0;
        return n.lo;
    }
    const int sh = msb > 52 ? msb - 52 : 0;
    uint64_t mant = shr128(n, sh).lo;
    int cmp = 0;                          // rest against half an ulp
    if (sh > 0) {
        const U128 back = shl128(shr128(n, sh), sh);
        U128 rest;
        rest.lo = n.lo - back.lo;
        rest.hi = n.hi - back.hi - (n.lo < back.lo ? 1u : 0u);
        U128 one;
        one.hi = 0; one.lo = 1;
        cmp = cmp128(rest, shl128(one, sh - 1));
        if (cmp == 0 && sticky) cmp = 1;
    } else {
        cmp = -1;                         // below half (only sticky bits)
    }
    int e = sh;
    if (cmp > 0 || (cmp == 0 && (mant & 1u))) {
        ++mant;
        if (mant >> 53) { mant >>= 1; ++e; }
    }
    *exp2 = e;
    return mant;
}

// 256-bit unsigned integer (little-endian words) for |e10| in 28..60
struct B4 {
    uint64_t w[4];
};
LBM_HD void b4_mul_small(B4& a, uint64_t m) {      // a *= m, m < 2^32, no overflow
    uint64_t carry = 0;
    for (int i = 0; i < 4; ++i) {
        const U128 p = mul64(a.w[i], m);
        const uint64_t lo = p.lo + carry;
        carry = p.hi + (lo < p.lo ? 1u : 0u);
        a.w[i] = lo;
    }
}
LBM_HD int b4_bitlen(const B4& a) {
    for (int i = 3; i >= 0; --i)
        if (a.w[i]) return 64 * i + 64 - clz64(a.w[i]);
    return 0;
}
LBM_HD int b4_bit(const B4& a, int i) { return (int)((a.w[i >> 6] >> (i & 63)) & 1u); }
LBM_HD bool b4_any_below(const B4& a, int i) {     // any bit < i set
    for (int k = 0; k < 4 && 64 * k < i; ++k) {
        const int n = i - 64 * k;
        const uint64_t m = n >= 64 ? ~0ull : ((1ull << n) - 1u);
        if (a.w[k] & m) return true;
    }
    return false;
}
LBM_HD uint64_t b4_bits(const B4& a, int lo, int n) {   // bits [lo, lo+n), n <= 64
    uint64_t r = 0;
    for (int i = n - 1; i >= 0; --i) r = (r << 1) | (uint64_t)b4_bit(a, lo + i);
    return r;
}
LBM_HD B4 b4_pow5(int k) {
    B4 d = {{1u, 0u, 0u, 0u}};
    for (int i = 0; i < k; ++i) b4_mul_small(d, 5u);
    return d;
}
LBM_HD int b4_cmp(const B4& a, const B4& b) {
    for (int i = 3; i >= 0; --i)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    return 0;
}
LBM_HD void b4_sub(B4& a, const B4& b) {           // a -= b, a >= b
    uint64_t borrow = 0;
    for (int i = 0; i < 4; ++i) {
        const uint64_t x = a.w[i], y = b.w[i];
        const uint64_t d = x - y - borrow;
        borrow = (x < y || (x == y && borrow)) ? 1u : 0u;
        a.w[i] = d;
    }
}
LBM_HD void b4_shl1_or(B4& a, int bit) {
    for (int i = 3; i > 0; --i) a.w[i] = (a.w[i] << 1) | (a.w[i - 1] >> 63);
    a.w[0] = (a.w[0] << 1) | (uint64_t)bit;
}

// exact w * 10^e10 (w != 0); false when outside the exact scope
LBM_HD bool exact_value(uint64_t w, int e10, double* out) {
    if (e10 > 60 || e10 < -60) return false;
    if (e10 >= 0 && e10 <= 27) {
        const U128 n = mul64(w, pow5(e10));
        int e2;
        const uint64_t m = round53(n, false, &e2);
        *out = scale2(m, e2 + e10);
        return true;
    }
    if (e10 > 27) {
        // N = w * 5^e10 (< 2^204), rounded to 53 bits by its bits
        B4 n = b4_pow5(e10);
        // multiply by w in two 32-bit halves: n * w = n * lo + (n * hi) << 32
        B4 a = n, b = n;
        b4_mul_small(a, w & 0xffffffffull);
        b4_mul_small(b, w >> 32);
        // a += b << 32
        uint64_t carry = 0;
        uint64_t prev = 0;
        for (int i = 0; i < 4; ++i) {
            const uint64_t sh = (b.w[i] << 32) | (prev >> 32);
            prev = b.w[i];
            const uint64_t s1 = a.w[i] + sh;
            const uint64_t c1 = s1 < sh ? 1u : 0u;
            const uint64_t s2 = s1 + carry;
            carry = c1 + (s2 < s1 ? 1u : 0u);
            a.w[i] = s2;
        }
        const int msb = b4_bitlen(a) - 1;
        const int sh = msb - 52;
        uint64_t mant = b4_bits(a, sh, 53);
        const bool half = b4_bit(a, sh - 1) != 0, below = b4_any_below(a, sh - 1);
        int e = sh;
        if (half && (below || (mant & 1u))) {
            ++mant;
            if (mant >> 53) { mant >>= 1; ++e; }
        }
        *out = scale2(mant, e + e10);
        return true;
    }
    const int k = -e10;
    if (k <= 27) {
        const uint64_t d = pow5(k);
        const int s = 64 + clz64(w);            // w << s has its top bit at 127
        U128 n;
        n.hi = w << (s - 64);
        n.lo = 0;
        // q = n / d: high word first (hi < 2^64, d < 2^63)
        const uint64_t qh = n.hi / d, rh = n.hi % d;
        uint64_t r;
        const uint64_t ql = div128_small(rh, n.lo, d, &r);
        U128 q;
        q.hi = qh; q.lo = ql;
        int e2;
        const uint64_t m = round53(q, r != 0, &e2);
        *out = scale2(m, e2 - s - k);
        return true;
    }
    // k in 28..60: q = floor(w 2^s / 5^k) by restoring division, s chosen
    // so that q has 56 or 57 bits; r != 0 is the sticky bit
    const B4 d = b4_pow5(k);
    const int wl = 64 - clz64(w);
    const int s = b4_bitlen(d) - wl + 56;
    B4 r = {{0u, 0u, 0u, 0u}};
    uint64_t q = 0;
    for (int i = wl + s - 1; i >= 0; --i) {
        const int bit = i >= s ? (int)((w >> (i - s)) & 1u) : 0;
        b4_shl1_or(r, bit);
        q <<= 1;
        if (b4_cmp(r, d) >= 0) { b4_sub(r, d); q |= 1u; }
    }
    const bool sticky = (r.w[0] | r.w[1] | r.w[2] | r.w[3]) != 0;
    U128 qq;
    qq.hi = 0; qq.lo = q;
    int e2;
    const uint64_t m = round53(qq, sticky, &e2);
    *out = scale2(m, e2 - s - k);
    return true;
}

// Parses one number at p (after skipping whitespace) with the prefix
// grammar of the host reader.  Returns the end pointer, or nullptr when no
// number starts there (the reader's parse failure).  *exact = false when
// the value is outside the exact scope (*out is then unset).
LBM_HD const char* parse_number(const char* p, const char* end, double* out, bool* exact) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) ++p;
    if (p >= end) return nullptr;
    bool neg = false;
    const char* q = p;
    if (*q == '+' || *q == '-') { neg = *q == '-'; ++q; }
    uint64_t w = 0;
    int nd = 0, d10 = 0;
    bool digits = false, lost = false;
    while (q < end && *q >= '0' && *q <= '9') {
        const int dg = *q - '0';
        digits = true;
        if (nd < 19) { if (w || dg) { w = w * 10u + (uint64_t)dg; if (w) ++nd; } }
        else { if (dg) lost = true; ++d10; }
        ++q;
    }
    if (q < end && *q == '.') {
        ++q;
        while (q < end && *q >= '0' && *q <= '9') {
            const int dg = *q - '0';
            digits = true;
            if (nd < 19) { if (w || dg) { w = w * 10u + (uint64_t)dg; if (w) ++nd; } --d10; }
            else if (dg) lost = true;
            ++q;
        }
    }
    if (!digits) return nullptr;
    if (q < end && (*q == 'e' || *q == 'E')) {
        const char* r = q + 1;
        bool eneg = false;
        if (r < end && (*r == '+' || *r == '-')) { eneg = *r == '-'; ++r; }
        if (r < end && *r >= '0' && *r <= '9') {
            int ev = 0;
            while (r < end && *r >= '0' && *r <= '9') {
                if (ev < 100000) ev = ev * 10 + (*r - '0');
                ++r;
            }
            d10 += eneg ? -ev : ev;
            q = r;
        }
    }
    if (w == 0) {
        *out = neg ? -0.0 : 0.0;
        *exact = true;
        return q;
    }
    double v;
    if (lost || !exact_value(w, d10, &v)) { *exact = false; return q; }
    *out = neg ? -v : v;
    *exact = true;
    return q;
}

}  // namespace stlnum
}  // namespace lbm
