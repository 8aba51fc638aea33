// Multi-word fixed-point arithmetic for the deep-zoom kernels.
//
// A number is N 32-bit words (N even: N/2 64-bit limbs), two's complement,
// least significant word first, with F = 32*N - 8 fractional bits: 1 sign
// bit, 7 integer bits.  The iteration only ever holds |values| < 8 before a
// square (larger ones have already escaped) so squares stay below 64 and
// |z|^2 below 128: the format never overflows.
//
// Products are computed on magnitudes with PTX carry chains
// (mad.lo.cc / madc.lo.cc / madc.hi.cc: one 32x32->64 partial product per
// two IMADs) and truncated: partial products that land entirely below
// column N-2 are skipped.  Their sum is below N^2 * 2^(32(N-2)+64), i.e.
// below N^2 * 2^-24 units of the result's last place, so the truncated
// product is within 2 ulp of floor(a*b / 2^F).
#pragma once

#include <stdint.h>

namespace mdz {
namespace fx {

// acc[k] holds product column (N-2+k), k = 0..N+1.
template <int N>
__device__ __forceinline__ void mul_trunc(const uint32_t (&a)[N], const uint32_t (&b)[N],
                                          uint32_t (&acc)[N + 2])
{
#pragma unroll
    for (int k = 0; k < N + 2; ++k)
        acc[k] = 0u;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        constexpr int base = N - 2;
        const int j0 = (base - i) > 0 ? (base - i) : 0;
        // low halves into columns i+j, carry into column i+N (zero so far)
#pragma unroll
        for (int j = j0; j < N; ++j) {
            if (j == j0)
                asm volatile("mad.lo.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j - base]) : "r"(a[i]), "r"(b[j]));
            else
                asm volatile("madc.lo.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j - base]) : "r"(a[i]), "r"(b[j]));
        }
        asm volatile("addc.u32 %0, 0, 0;" : "=r"(acc[i + 2]));
        // high halves into columns i+j+1; the final carry is provably zero
#pragma unroll
        for (int j = j0; j < N; ++j) {
            if (j == j0)
                asm volatile("mad.hi.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j + 1 - base]) : "r"(a[i]), "r"(b[j]));
            else if (j < N - 1)
                asm volatile("madc.hi.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j + 1 - base]) : "r"(a[i]), "r"(b[j]));
            else
                asm volatile("madc.hi.u32 %0, %1, %2, %0;" : "+r"(acc[i + j + 1 - base]) : "r"(a[i]), "r"(b[j]));
        }
    }
}

// Truncated square of a magnitude; acc as in mul_trunc.
template <int N>
__device__ __forceinline__ void sqr_trunc(const uint32_t (&a)[N], uint32_t (&acc)[N + 2])
{
    constexpr int base = N - 2;
#pragma unroll
    for (int k = 0; k < N + 2; ++k)
        acc[k] = 0u;
    // off-diagonal products a_i a_j, i < j
#pragma unroll
    for (int i = 0; i < N - 1; ++i) {
        const int jl = (i + 1) > (base - i) ? (i + 1) : (base - i);
        if (jl > N - 1)
            continue;
#pragma unroll
        for (int j = jl; j < N; ++j) {
            if (j == jl)
                asm volatile("mad.lo.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j - base]) : "r"(a[i]), "r"(a[j]));
            else
                asm volatile("madc.lo.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j - base]) : "r"(a[i]), "r"(a[j]));
        }
        asm volatile("addc.u32 %0, 0, 0;" : "=r"(acc[i + 2]));
#pragma unroll
        for (int j = jl; j < N; ++j) {
            if (j == jl)
                asm volatile("mad.hi.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j + 1 - base]) : "r"(a[i]), "r"(a[j]));
            else if (j < N - 1)
                asm volatile("madc.hi.cc.u32 %0, %1, %2, %0;" : "+r"(acc[i + j + 1 - base]) : "r"(a[i]), "r"(a[j]));
            else
                asm volatile("madc.hi.u32 %0, %1, %2, %0;" : "+r"(acc[i + j + 1 - base]) : "r"(a[i]), "r"(a[j]));
        }
    }
    // double
#pragma unroll
    for (int k = N + 1; k > 0; --k)
        acc[k] = __funnelshift_l(acc[k - 1], acc[k], 1);
    acc[0] <<= 1;
    // diagonal a_i^2 into columns 2i, 2i+1 (one carry chain)
    constexpr int i0 = (base - 1) > 0 ? (base - 1 + 1) / 2 : 0;  // first i with 2i+1 >= base
    bool first = true;
#pragma unroll
    for (int i = i0; i < N; ++i) {
        if (2 * i >= base) {
            if (first)
                asm volatile("mad.lo.cc.u32 %0, %1, %1, %0;" : "+r"(acc[2 * i - base]) : "r"(a[i]));
            else
                asm volatile("madc.lo.cc.u32 %0, %1, %1, %0;" : "+r"(acc[2 * i - base]) : "r"(a[i]));
            first = false;
        }
        if (first)
            asm volatile("mad.hi.cc.u32 %0, %1, %1, %0;" : "+r"(acc[2 * i + 1 - base]) : "r"(a[i]));
        else if (i < N - 1)
            asm volatile("madc.hi.cc.u32 %0, %1, %1, %0;" : "+r"(acc[2 * i + 1 - base]) : "r"(a[i]));
        else
            asm volatile("madc.hi.u32 %0, %1, %1, %0;" : "+r"(acc[2 * i + 1 - base]) : "r"(a[i]));
        first = false;
    }
}

// r = acc >> (F - s) restricted to N words: SH = 24 gives floor(P / 2^F),
// SH = 23 gives floor(2P / 2^F).
template <int N, int SH>
__device__ __forceinline__ void extract(const uint32_t (&acc)[N + 2], uint32_t (&r)[N])
{
#pragma unroll
    for (int k = 0; k < N; ++k)
        r[k] = __funnelshift_r(acc[1 + k], acc[2 + k], SH);
}

// r = c + (x ^ m) + (m & 1): c + x when m == 0, c - x when m == ~0.
template <int N, class CGet>
__device__ __forceinline__ void add_signed(const CGet& c, const uint32_t (&x)[N], uint32_t m,
                                           uint32_t (&r)[N])
{
    uint32_t dummy;
    asm volatile("add.cc.u32 %0, %1, 0xffffffff;" : "=r"(dummy) : "r"(m & 1u));
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k < N - 1)
            asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(r[k]) : "r"(c(k)), "r"(x[k] ^ m));
        else
            asm volatile("addc.u32 %0, %1, %2;" : "=r"(r[k]) : "r"(c(k)), "r"(x[k] ^ m));
    }
    (void)dummy;
}

// r = a - b
template <int N>
__device__ __forceinline__ void sub(const uint32_t (&a)[N], const uint32_t (&b)[N], uint32_t (&r)[N])
{
    asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(r[0]) : "r"(a[0]), "r"(b[0]));
#pragma unroll
    for (int k = 1; k < N; ++k) {
        if (k < N - 1)
            asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(r[k]) : "r"(a[k]), "r"(b[k]));
        else
            asm volatile("subc.u32 %0, %1, %2;" : "=r"(r[k]) : "r"(a[k]), "r"(b[k]));
    }
}

// In place |x|; returns the sign mask (0 or ~0) of the input.
template <int N>
__device__ __forceinline__ uint32_t abs_inplace(uint32_t (&x)[N])
{
    const uint32_t m = (uint32_t)((int32_t)x[N - 1] >> 31);
    uint32_t dummy;
    asm volatile("add.cc.u32 %0, %1, 0xffffffff;" : "=r"(dummy) : "r"(m & 1u));
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k < N - 1)
            asm volatile("addc.cc.u32 %0, %1, 0;" : "=r"(x[k]) : "r"(x[k] ^ m));
        else
            asm volatile("addc.u32 %0, %1, 0;" : "=r"(x[k]) : "r"(x[k] ^ m));
    }
    (void)dummy;
    return m;
}

// |x| >= 8 (conservative on the negative side by less than 2^-24): the
// value has certainly escaped, and squaring it could overflow.
template <int N>
__device__ __forceinline__ bool big(const uint32_t (&x)[N])
{
    const int32_t top = (int32_t)x[N - 1];
    return top >= 0x08000000 || top < -0x08000000;
}

// a + b > 4 for non-negative a, b (< 64 each).
template <int N>
__device__ __forceinline__ bool sum_gt4(const uint32_t (&a)[N], const uint32_t (&b)[N])
{
    uint32_t s[N];
    asm volatile("add.cc.u32 %0, %1, %2;" : "=r"(s[0]) : "r"(a[0]), "r"(b[0]));
#pragma unroll
    for (int k = 1; k < N; ++k) {
        if (k < N - 1)
            asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(s[k]) : "r"(a[k]), "r"(b[k]));
        else
            asm volatile("addc.u32 %0, %1, %2;" : "=r"(s[k]) : "r"(a[k]), "r"(b[k]));
    }
    uint32_t low = 0;
#pragma unroll
    for (int k = 0; k < N - 1; ++k)
        low |= s[k];
    const uint32_t top = s[N - 1];
    return top > 0x04000000u || (top == 0x04000000u && low != 0u);
}

}  // namespace fx
}  // namespace mdz
