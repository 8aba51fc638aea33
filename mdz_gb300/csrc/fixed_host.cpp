// Host-side conversions between MPFR / GMP values and the kernels'
// fixed-point format (32-bit words, two's complement, least significant
// first, F = 32*words - 8 fractional bits).
//
// These replace, on the host, the reference's per-pixel MPFR coordinate
// arithmetic (src/fractal.c:159-192): the GPU gets exact fixed-point x[ix]
// and y[line] tables instead of recomputing them with rounded MPFR calls.
#include <limits.h>
#include <math.h>
#include <stdarg.h>
#include <string.h>

#include <vector>

#include "internal.h"

namespace mdz {

namespace {

// Shift the magnitude given by `limbs` (value = M * 2^(shift)) into the
// fixed-point words: out = floor(M * 2^shift) (truncated toward zero).
int place_magnitude(const uint64_t* limbs, int n, long shift, int words, uint32_t* out)
{
    memset(out, 0, sizeof(uint32_t) * words);
    const long total_bits = 32L * words;
    for (int i = 0; i < n; ++i) {
        const uint64_t limb = limbs[i];
        if (!limb)
            continue;
        for (int b = 0; b < 64; ++b) {
            if (!((limb >> b) & 1u))
                continue;
            const long pos = (long)i * 64 + b + shift;
            if (pos < 0)
                continue;  // below the last fractional bit: truncated
            if (pos >= total_bits - 1)
                return MDZGPU_ERR_RANGE;
            out[pos / 32] |= 1u << (pos % 32);
        }
    }
    return MDZGPU_OK;
}

void negate(uint32_t* x, int words)
{
    uint64_t carry = 1;
    for (int k = 0; k < words; ++k) {
        const uint64_t v = (uint64_t)(~x[k]) + carry;
        x[k] = (uint32_t)v;
        carry = v >> 32;
    }
}

bool fits_coordinate(const uint32_t* x, int words)
{
    // |x| < 4: top word in (-4<<24, 4<<24)
    const int32_t top = (int32_t)x[words - 1];
    return top < (4 << 24) && top >= -(4 << 24);
}

}  // namespace

int fx_from_mpval(const mdzgpu_mpval* v, int words, uint32_t* out)
{
    if (!v || !v->d || v->nlimbs <= 0) {
        memset(out, 0, sizeof(uint32_t) * words);
        return MDZGPU_OK;
    }
    // value = sign * M * 2^(exp - 64 n); fixed = value * 2^F
    const long F = 32L * words - 8;
    const long shift = (long)v->exp - 64L * v->nlimbs + F;
    int rc = place_magnitude(v->d, v->nlimbs, shift, words, out);
    if (rc)
        return rc;
    if (v->sign < 0)
        negate(out, words);
    return MDZGPU_OK;
}

int fx_from_mpfr(const mdz_mpfr* v, int words, uint32_t* out)
{
    if (v->exp == MDZ_MPFR_EXP_ZERO) {
        memset(out, 0, sizeof(uint32_t) * words);
        return MDZGPU_OK;
    }
    if (v->exp == MDZ_MPFR_EXP_NAN || v->exp == MDZ_MPFR_EXP_INF)
        return MDZGPU_ERR_RANGE;
    mdzgpu_mpval m;
    m.sign = v->sign < 0 ? -1 : 1;
    m.nlimbs = (int32_t)((v->prec + 63) / 64);
    m.exp = v->exp;
    m.d = v->d;
    return fx_from_mpval(&m, words, out);
}

int fx_from_mpf(const mdz_mpf* v, int words, uint32_t* out)
{
    const int n = v->size < 0 ? -v->size : v->size;
    if (n == 0) {
        memset(out, 0, sizeof(uint32_t) * words);
        return MDZGPU_OK;
    }
    // value = sum d[i] 2^(64 (i - n + exp))  -> M * 2^(64 (exp - n))
    const long F = 32L * words - 8;
    const long shift = 64L * ((long)v->exp - n) + F;
    int rc = place_magnitude(v->d, n, shift, words, out);
    if (rc)
        return rc;
    if (v->size < 0)
        negate(out, words);
    return MDZGPU_OK;
}

double fx_to_double(const uint32_t* x, int words)
{
    std::vector<uint32_t> m(x, x + words);
    double sign = 1.0;
    if ((int32_t)m[words - 1] < 0) {
        negate(m.data(), words);
        sign = -1.0;
    }
    double v = 0.0;
    for (int k = words - 1; k >= 0; --k)
        v = v * 4294967296.0 + m[k];
    return sign * ldexp(v, -(32 * words - 8));
}

// out = a + sign * floor(k * step / div), computed exactly on magnitudes.
void fx_affine(const uint32_t* a, const uint32_t* step, long k, long div, int sign,
               int words, uint32_t* out)
{
    std::vector<uint32_t> s(step, step + words);
    bool neg = false;
    if ((int32_t)s[words - 1] < 0) {
        negate(s.data(), words);
        neg = true;
    }
    // p = s * k  (one extra word)
    std::vector<uint32_t> p(words + 1, 0);
    uint64_t carry = 0;
    for (int i = 0; i < words; ++i) {
        const unsigned __int128 v = (unsigned __int128)s[i] * (uint64_t)k + carry;
        p[i] = (uint32_t)v;
        carry = (uint64_t)(v >> 32);
    }
    p[words] = (uint32_t)carry;
    // q = p / div
    unsigned __int128 rem = 0;
    for (int i = words; i >= 0; --i) {
        const unsigned __int128 cur = (rem << 32) | p[i];
        p[i] = (uint32_t)(cur / (uint64_t)div);
        rem = cur % (uint64_t)div;
    }
    if (neg)
        sign = -sign;
    // out = a +/- q (mod 2^(32 words))
    std::vector<uint32_t> q(p.begin(), p.begin() + words);
    if (sign < 0)
        negate(q.data(), words);
    uint64_t c = 0;
    for (int i = 0; i < words; ++i) {
        const uint64_t v = (uint64_t)a[i] + q[i] + c;
        out[i] = (uint32_t)v;
        c = v >> 32;
    }
}

bool fx_fits_coordinate(const uint32_t* x, int words)
{
    return fits_coordinate(x, words);
}

// mpfr_get_d(x, MPFR_RNDN) for a regular value: round the mantissa to 53
// bits, ties to even (the rounding mpfr_get_ld performs when long double is
// IEEE double, src/fractal.c:50-52).
double mpfr_to_double_rn(const mdz_mpfr* v)
{
    if (v->exp == MDZ_MPFR_EXP_ZERO)
        return v->sign < 0 ? -0.0 : 0.0;
    if (v->exp == MDZ_MPFR_EXP_NAN)
        return NAN;
    if (v->exp == MDZ_MPFR_EXP_INF)
        return v->sign < 0 ? -INFINITY : INFINITY;
    const int n = (int)((v->prec + 63) / 64);
    const uint64_t top = v->d[n - 1];  // value = top * 2^(exp - 64) + lower limbs
    // bits of `top` dropped so that the kept part has 53 bits, or fewer
    // when the result is subnormal (quantum 2^-1074)
    long drop = 11;
    if (-1074 - (v->exp - 64) > drop)
        drop = -1074 - (v->exp - 64);
    bool sticky = false;
    for (int i = n - 2; i >= 0 && !sticky; --i)
        sticky = v->d[i] != 0;
    uint64_t kept, rb;
    if (drop >= 65) {
        kept = 0;
        rb = 0;
        sticky = sticky || top != 0;
    } else if (drop == 64) {
        kept = 0;
        rb = top >> 63;
        sticky = sticky || (top & ~(1ull << 63)) != 0;
    } else {
        kept = top >> drop;
        rb = (top >> (drop - 1)) & 1u;
        sticky = sticky || (top & ((1ull << (drop - 1)) - 1)) != 0;
    }
    if (rb && (sticky || (kept & 1u)))
        kept += 1;  // may carry to 2^53: still exact in a double
    const double r = ldexp((double)kept, (int)(v->exp - 64 + drop));
    return v->sign < 0 ? -r : r;
}

int mp_words_for_precision(long precision)
{
    long bits = precision + 8;
    long words = (bits + 31) / 32;
    if (words & 1)
        ++words;  // whole 64-bit limbs
    if (words < 4)
        words = 4;
    return (int)words;
}

}  // namespace mdz
