// Exact "%24.16e" formatting of an FP32 value (promoted to double, as the
// reference's sprintf calls in FSSW::combine_samples_to_OSCAR do,
// src/FSSW.cpp:472-482), with integer arithmetic only, for host and device.
//
// A finite float is v = m * 2^e with m < 2^24.  With p = floor(log10 |v|) the
// 17 significant digits are D = round(|v| * 10^(16 - p)), rounded to nearest
// with ties to even (the C library's behaviour in the default rounding mode):
//   * b = 16 - p >= 0: |v| 10^b = m 5^b 2^(e + b); m 5^b has at most 166 bits
//     (b <= 61 for floats), held in three 64-bit limbs, then shifted right by
//     -(e + b) when that is negative;
//   * b < 0 (|v| >= 1e17, so e >= 33 and e + b > 0): |v| 10^b = m 2^(e+b) / 5^-b
//     with m 2^(e+b) < 2^128 and 5^-b < 2^52: one 128 / 64 division.
// p comes from the binary exponent and is corrected by one when D lands
// outside [10^16, 10^17).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define FMT_HD __host__ __device__ __forceinline__
#else
#define FMT_HD inline
#endif

namespace iss {
namespace fmt {

struct U192 {
    uint64_t w[3];   // little-endian limbs
};

FMT_HD void mul_small(U192& a, uint64_t f) {
    unsigned __int128 carry = 0;
    for (int i = 0; i < 3; i++) {
        const unsigned __int128 t = static_cast<unsigned __int128>(a.w[i]) * f + carry;
        a.w[i] = static_cast<uint64_t>(t);
        carry = t >> 64;
    }
}

// a >> s, with the rounding information of the bits shifted out:
// *half = the highest dropped bit, *sticky = any lower dropped bit
FMT_HD U192 shr_round(const U192& a, int s, int* half, int* sticky) {
    U192 r = {{0, 0, 0}};
    *half = 0;
    *sticky = 0;
    if (s <= 0) return a;
    // half bit: bit s-1; sticky: bits 0 .. s-2
    const int hb = s - 1;
    if (hb < 192) *half = static_cast<int>((a.w[hb >> 6] >> (hb & 63)) & 1u);
    for (int i = 0; i < 3; i++) {
        const int lo = i * 64;
        if (lo >= hb) break;
        const int n = hb - lo;   // bits of limb i below the half bit
        const uint64_t mask = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
        if (a.w[i] & mask) *sticky = 1;
    }
    const int ws = s >> 6, bs = s & 63;
    for (int i = 0; i < 3; i++) {
        const int j = i + ws;
        uint64_t v = 0;
        if (j < 3) {
            v = a.w[j] >> bs;
            if (bs && j + 1 < 3) v |= a.w[j + 1] << (64 - bs);
        }
        r.w[i] = v;
    }
    return r;
}

// D = round_half_even(|v| * 10^(16 - p)) for |v| = m 2^e, m > 0
FMT_HD uint64_t scaled_digits(uint32_t m, int e, int p) {
    const int b = 16 - p;
    const int a = e + b;
    if (b >= 0) {
        U192 x = {{m, 0, 0}};
        int k = b;
        while (k >= 27) {   // 5^27 < 2^63
            mul_small(x, 7450580596923828125ull);
            k -= 27;
        }
        uint64_t f = 1;
        for (int i = 0; i < k; i++) f *= 5;
        mul_small(x, f);
        if (a >= 0) {
            // |v| 10^b is an integer; below 10^17 whenever p is right, so a
            // result of 64 bits or more only says that p is too small
            if (x.w[1] || x.w[2] || a >= 64) return ~0ull;
            if (a > 0 && (x.w[0] >> (64 - a))) return ~0ull;
            return x.w[0] << a;
        }
        int half, sticky;
        U192 q = shr_round(x, -a, &half, &sticky);
        if (q.w[1] || q.w[2]) return ~0ull;
        uint64_t d = q.w[0];
        if (half && (sticky || (d & 1))) d++;
        return d;
    }
    // b < 0: m 2^a / 5^-b with a > 0
    uint64_t den = 1;
    for (int i = 0; i < -b; i++) den *= 5;
    if (a >= 128 - 24) return ~0ull;
    const unsigned __int128 num = static_cast<unsigned __int128>(m) << a;
    const unsigned __int128 q = num / den;
    const uint64_t r = static_cast<uint64_t>(num - q * den);
    if (q >> 64) return ~0ull;
    uint64_t d = static_cast<uint64_t>(q);
    const uint64_t twice = 2 * r;   // r < den < 2^52: no overflow
    if (twice > den || (twice == den && (d & 1))) d++;
    return d;
}

// Writes exactly 24 characters (no terminator): printf("%24.16e", (double)x).
FMT_HD void format_e24_16(float x, char* out) {
    uint32_t bits;
#if defined(__CUDA_ARCH__)
    bits = __float_as_uint(x);
#else
    __builtin_memcpy(&bits, &x, 4);
#endif
    const int neg = static_cast<int>(bits >> 31);
    const int ex = static_cast<int>((bits >> 23) & 0xFFu);
    uint32_t m = bits & 0x7FFFFFu;
    char buf[24];
    int len = 0;
    if (ex == 0xFF) {
        const char* s = m ? "nan" : "inf";
        if (neg) buf[len++] = '-';
        for (int i = 0; i < 3; i++) buf[len++] = s[i];
    } else {
        int e;
        if (ex) {
            m |= 0x800000u;
            e = ex - 150;
        } else {
            e = -149;
        }
        uint64_t D = 0;
        int p = 0;
        if (m != 0) {
            // estimate p = floor(log10(m 2^e)) from the bit length
            int nb = 0;
            for (uint32_t t = m; t; t >>= 1) nb++;
            const int e2 = e + nb - 1;                     // 2^e2 <= |v| < 2^(e2+1)
            p = (e2 >= 0) ? (e2 * 78913) >> 18 : -(((-e2) * 78913 + 262143) >> 18);
            for (int it = 0; it < 4; it++) {
                D = scaled_digits(m, e, p);
                if (D >= 100000000000000000ull) {
                    p++;
                } else if (D < 10000000000000000ull) {
                    p--;
                } else {
                    break;
                }
            }
            if (D == 100000000000000000ull) {   // rounding carried into a new digit
                D = 10000000000000000ull;
                p++;
            }
        }
        char dig[17];
        for (int i = 16; i >= 0; i--) {
            dig[i] = static_cast<char>('0' + D % 10);
            D /= 10;
        }
        if (neg) buf[len++] = '-';
        buf[len++] = dig[0];
        buf[len++] = '.';
        for (int i = 1; i < 17; i++) buf[len++] = dig[i];
        buf[len++] = 'e';
        buf[len++] = p < 0 ? '-' : '+';
        const int ap = p < 0 ? -p : p;
        if (ap >= 100) buf[len++] = static_cast<char>('0' + ap / 100);
        buf[len++] = static_cast<char>('0' + (ap / 10) % 10);
        buf[len++] = static_cast<char>('0' + ap % 10);
    }
    const int pad = 24 - len;
    for (int i = 0; i < pad; i++) out[i] = ' ';
    for (int i = 0; i < len; i++) out[pad + i] = buf[i];
}

// Right-aligned decimal integer in `width` characters (std::setw(width) << v).
FMT_HD void format_int(long long v, int width, char* out) {
    char buf[24];
    int len = 0;
    unsigned long long a = v < 0 ? 0ull - static_cast<unsigned long long>(v)
                                 : static_cast<unsigned long long>(v);
    do {
        buf[len++] = static_cast<char>('0' + a % 10);
        a /= 10;
    } while (a);
    if (v < 0) buf[len++] = '-';
    int pos = 0;
    for (int i = len; i < width; i++) out[pos++] = ' ';
    for (int i = len - 1; i >= 0; i--) out[pos++] = buf[i];
}

// Characters format_int writes for v at `width`.
FMT_HD int int_width(long long v, int width) {
    int len = v < 0 ? 1 : 0;
    unsigned long long a = v < 0 ? 0ull - static_cast<unsigned long long>(v)
                                 : static_cast<unsigned long long>(v);
    do {
        len++;
        a /= 10;
    } while (a);
    return len > width ? len : width;
}

}  // namespace fmt
}  // namespace iss
