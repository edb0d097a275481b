// A coordinate rounded through the grid file's text form: the double that
// strtod returns for printf("%.16f", v).  The grid generators store their
// coordinates this way so that an in-memory grid is bit-identical to the same
// grid written out and read back (src/mesh.cpp:4016-4089 reads degrees as
// text).
//
// Exact integer arithmetic in place of the C library's conversions, so that the
// device generator gives the same values as the host one:
//   1. N = |v| * 10^16 rounded to an integer, ties to even (printf's rounding of
//      the 16th decimal in round-to-nearest mode), with |v| = m 2^e exactly
//      and m 10^16 held in 128 bits;
//   2. the double nearest N / 10^16, ties to even (strtod): a 53-bit quotient
//      of N 2^k / 10^16 with the remainder deciding the last bit.
// For |v| >= 1 the 16 decimals resolve v to better than half its last bit, so
// the round trip returns v itself; only |v| < 1 changes.
#pragma once

#include <cstdint>
#include <cstring>

#ifndef ODIS_HD
#ifdef __CUDACC__
#define ODIS_HD __host__ __device__
#else
#define ODIS_HD
#endif
#endif

namespace odis {

ODIS_HD inline uint64_t text_bits(double v)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    std::memcpy(&b, &v, 8);
    return b;
#endif
}

ODIS_HD inline double text_double(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double v;
    std::memcpy(&v, &b, 8);
    return v;
#endif
}

ODIS_HD inline int text_bitlen(unsigned __int128 x)
{
    int n = 0;
    while (x) { x >>= 1; n++; }
    return n;
}

ODIS_HD inline double text_round16(double v)
{
    const uint64_t bits = text_bits(v);
    const uint64_t sign = bits & 0x8000000000000000ull;
    const int bexp = (int)((bits >> 52) & 0x7ff);
    uint64_t m = bits & 0x000fffffffffffffull;
    if (bexp == 0x7ff) return v;                      // inf / nan
    if (bexp == 0 && m == 0) return v;                // +-0 prints and parses as itself
    if (bexp >= 1023) return v;                       // |v| >= 1: the round trip is exact
    int e;                                            // |v| = m 2^e
    if (bexp == 0) e = -1074;
    else { m |= 1ull << 52; e = bexp - 1075; }
    const uint64_t kTen16 = 10000000000000000ull;
    // 1. N = round_half_even(m 10^16 / 2^-e)
    const unsigned __int128 num = (unsigned __int128)m * kTen16;   // < 2^107
    const int sh = -e;
    uint64_t N;
    if (sh > 120) {
        N = 0;                                        // |v| 10^16 < 2^-13
    } else {
        const unsigned __int128 q = num >> sh;
        const unsigned __int128 rem = num - (q << sh);
        const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        N = (uint64_t)q;
        if (rem > half || (rem == half && (N & 1))) N++;
    }
    if (N == 0) return text_double(sign);             // "-0.0000000000000000" parses as -0.0
    // 2. nearest double to N / 10^16: M = floor(N 2^k / 10^16) in [2^52, 2^53)
    int k = 106 - text_bitlen((unsigned __int128)N);  // N 2^k < 2^107 (fits in 128 bits)
    unsigned __int128 M, R;
    for (;;) {
        const unsigned __int128 x = (unsigned __int128)N << k;
        M = x / kTen16;
        R = x - M * kTen16;
        if (M >= ((unsigned __int128)1 << 53)) { k--; continue; }
        if (M < ((unsigned __int128)1 << 52)) { k++; continue; }
        break;
    }
    const unsigned __int128 twoR = R * 2;
    if (twoR > kTen16 || (twoR == kTen16 && (M & 1))) M++;
    if (M == ((unsigned __int128)1 << 53)) { M >>= 1; k--; }
    const int be = 1023 + 52 - k;                     // M 2^-k, normal for N >= 1
    return text_double(sign | ((uint64_t)be << 52) | ((uint64_t)M & 0x000fffffffffffffull));
}

}  // namespace odis
