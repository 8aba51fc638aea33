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

#include <algorithm>
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
    // 8 integer/sign bits, and 32 bits beyond the precision so that every
    // p-bit coordinate with |x| >= 2^-32 converts exactly
    long bits = precision + 40;
    long words = (bits + 31) / 32;
    if (words & 1)
        ++words;  // whole 64-bit limbs
    if (words < 4)
        words = 4;
    return (int)words;
}

}  // namespace mdz

// ---------------------------------------------------------------------------
// p-bit binary floating point with round-to-nearest-even, for the pixel
// coordinates of the MPFR path.  fractal_mpfr_calculate_line
// (src/fractal.c:167-186) computes, each step rounded to img->precision bits:
//   y = ymax - (width / W) * line
//   x = (ix / W) * width + xmin
// The same roundings here give the kernel the very c values MPFR iterates.
// ---------------------------------------------------------------------------
namespace mdz {
namespace {

using Big = std::vector<uint32_t>;  // little-endian magnitude

struct BF {
    int sign = 1;   // +1 / -1
    Big m;          // magnitude; empty = zero
    long e = 0;     // value = sign * m * 2^e
};

void trim(Big& a)
{
    while (!a.empty() && a.back() == 0)
        a.pop_back();
}

long bitlen(const Big& a)
{
    if (a.empty())
        return 0;
    return 32L * (long)(a.size() - 1) + (32 - __builtin_clz(a.back()));
}

bool bit(const Big& a, long i)
{
    if (i < 0 || i / 32 >= (long)a.size())
        return false;
    return (a[i / 32] >> (i % 32)) & 1u;
}

bool any_below(const Big& a, long i)  // any bit in [0, i)
{
    for (long w = 0; w * 32 < i && w < (long)a.size(); ++w) {
        uint32_t v = a[w];
        if ((w + 1) * 32 > i)
            v &= (i % 32) ? ((1u << (i % 32)) - 1) : 0xffffffffu;
        if (v)
            return true;
    }
    return false;
}

Big shr(const Big& a, long s)
{
    Big r;
    if (s <= 0)
        return a;
    const long ws = s / 32, bs = s % 32;
    for (long i = ws; i < (long)a.size(); ++i) {
        uint64_t v = a[i] >> bs;
        if (bs && i + 1 < (long)a.size())
            v |= (uint64_t)a[i + 1] << (32 - bs);
        r.push_back((uint32_t)v);
    }
    trim(r);
    return r;
}

Big shl(const Big& a, long s)
{
    if (a.empty())
        return a;
    const long ws = s / 32, bs = s % 32;
    Big r(ws, 0);
    uint32_t carry = 0;
    for (uint32_t w : a) {
        r.push_back((w << bs) | carry);
        carry = bs ? (w >> (32 - bs)) : 0;
    }
    if (carry)
        r.push_back(carry);
    trim(r);
    return r;
}

Big add_mag(const Big& a, const Big& b)
{
    Big r(std::max(a.size(), b.size()) + 1, 0);
    uint64_t c = 0;
    for (size_t i = 0; i < r.size(); ++i) {
        uint64_t v = c;
        if (i < a.size())
            v += a[i];
        if (i < b.size())
            v += b[i];
        r[i] = (uint32_t)v;
        c = v >> 32;
    }
    trim(r);
    return r;
}

int cmp_mag(const Big& a, const Big& b)
{
    if (a.size() != b.size())
        return a.size() < b.size() ? -1 : 1;
    for (size_t i = a.size(); i-- > 0;)
        if (a[i] != b[i])
            return a[i] < b[i] ? -1 : 1;
    return 0;
}

Big sub_mag(const Big& a, const Big& b)  // a >= b
{
    Big r(a.size(), 0);
    int64_t br = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        int64_t v = (int64_t)a[i] - br - (i < b.size() ? (int64_t)b[i] : 0);
        br = v < 0;
        r[i] = (uint32_t)(v + (br ? (1LL << 32) : 0));
    }
    trim(r);
    return r;
}

Big mul_mag(const Big& a, const Big& b)
{
    if (a.empty() || b.empty())
        return Big();
    Big r(a.size() + b.size(), 0);
    for (size_t i = 0; i < a.size(); ++i) {
        uint64_t c = 0;
        for (size_t j = 0; j < b.size(); ++j) {
            uint64_t v = (uint64_t)a[i] * b[j] + r[i + j] + c;
            r[i + j] = (uint32_t)v;
            c = v >> 32;
        }
        size_t k = i + b.size();
        while (c) {
            uint64_t v = (uint64_t)r[k] + c;
            r[k++] = (uint32_t)v;
            c = v >> 32;
        }
    }
    trim(r);
    return r;
}

// a / d (d small), remainder returned through rem
Big div_small(const Big& a, uint64_t d, uint64_t& rem)
{
    Big q(a.size(), 0);
    unsigned __int128 r = 0;
    for (size_t i = a.size(); i-- > 0;) {
        const unsigned __int128 cur = (r << 32) | a[i];
        q[i] = (uint32_t)(cur / d);
        r = cur % d;
    }
    trim(q);
    rem = (uint64_t)r;
    return q;
}

// Round to p significant bits, ties to even; `sticky` = nonzero bits were
// already dropped below the current last bit.
BF round_p(BF x, long p, bool sticky = false)
{
    trim(x.m);
    const long b = bitlen(x.m);
    if (b == 0)
        return x;
    if (b <= p && !sticky)
        return x;
    if (b <= p) {
        // only a sticky tail below the last bit: below half an ulp of a
        // p-bit value when b < p; at b == p the value is exact
        return x;
    }
    const long s = b - p;
    const bool rb = bit(x.m, s - 1);
    const bool st = sticky || any_below(x.m, s - 1);
    Big keep = shr(x.m, s);
    if (rb && (st || (!keep.empty() && (keep[0] & 1u)))) {
        keep = add_mag(keep, Big{1});
    }
    x.m = keep;
    x.e += s;
    if (bitlen(x.m) > p) {
        x.m = shr(x.m, 1);
        x.e += 1;
    }
    return x;
}

BF bf_add(const BF& a, const BF& b, long p)
{
    if (a.m.empty())
        return round_p(b, p);
    if (b.m.empty())
        return round_p(a, p);
    const long e = std::min(a.e, b.e);
    const Big am = shl(a.m, a.e - e), bm = shl(b.m, b.e - e);
    BF r;
    r.e = e;
    if (a.sign == b.sign) {
        r.m = add_mag(am, bm);
        r.sign = a.sign;
    } else {
        const int c = cmp_mag(am, bm);
        if (c == 0)
            return BF();
        r.m = c > 0 ? sub_mag(am, bm) : sub_mag(bm, am);
        r.sign = c > 0 ? a.sign : b.sign;
    }
    return round_p(r, p);
}

BF bf_mul(const BF& a, const BF& b, long p)
{
    BF r;
    r.m = mul_mag(a.m, b.m);
    r.e = a.e + b.e;
    r.sign = a.sign * b.sign;
    return round_p(r, p);
}

BF bf_mul_si(const BF& a, long k, long p)
{
    BF b;
    b.sign = k < 0 ? -1 : 1;
    const uint64_t u = (uint64_t)(k < 0 ? -k : k);
    if (u) {
        b.m = Big{(uint32_t)u, (uint32_t)(u >> 32)};
        trim(b.m);
    }
    return bf_mul(a, b, p);
}

// a / d for a small positive integer d, rounded to p bits
BF bf_div_si(const BF& a, long d, long p)
{
    if (a.m.empty())
        return a;
    // scale so that the quotient has at least p + 2 bits
    const long extra = p + 66;
    BF r;
    uint64_t rem = 0;
    r.m = div_small(shl(a.m, extra), (uint64_t)d, rem);
    r.e = a.e - extra;
    r.sign = a.sign;
    return round_p(r, p, rem != 0);
}

BF bf_from_mpval(const mdzgpu_mpval* v)
{
    BF r;
    if (!v || !v->d || v->nlimbs <= 0)
        return r;
    r.sign = v->sign < 0 ? -1 : 1;
    for (int i = 0; i < v->nlimbs; ++i) {
        r.m.push_back((uint32_t)v->d[i]);
        r.m.push_back((uint32_t)(v->d[i] >> 32));
    }
    trim(r.m);
    r.e = (long)v->exp - 64L * v->nlimbs;
    return r;
}

BF bf_from_int(long k)
{
    BF r;
    r.sign = k < 0 ? -1 : 1;
    const uint64_t u = (uint64_t)(k < 0 ? -k : k);
    r.m = Big{(uint32_t)u, (uint32_t)(u >> 32)};
    trim(r.m);
    return r;
}

// value * 2^F truncated toward zero into `words` two's complement words
int bf_to_fixed(const BF& x, int words, uint32_t* out)
{
    memset(out, 0, sizeof(uint32_t) * words);
    if (x.m.empty())
        return MDZGPU_OK;
    const long F = 32L * words - 8;
    const long sh = x.e + F;
    const Big v = sh >= 0 ? shl(x.m, sh) : shr(x.m, -sh);
    if (bitlen(v) >= 32L * words - 1)
        return MDZGPU_ERR_RANGE;
    for (size_t i = 0; i < v.size() && i < (size_t)words; ++i)
        out[i] = v[i];
    if (x.sign < 0)
        negate(out, words);
    return MDZGPU_OK;
}

}  // namespace

int mpfr_coordinate_tables(const mdzgpu_mpval* xmin, const mdzgpu_mpval* ymax,
                           const mdzgpu_mpval* width, int W, int row0, int nrows, long p,
                           int words, uint32_t* xs, uint32_t* ys)
{
    const BF bx = bf_from_mpval(xmin), by = bf_from_mpval(ymax), bw = bf_from_mpval(width);
    // img_xmin / width are copies at precision p (mpfr_set, src/fractal.c:161-162)
    const BF xm = round_p(bx, p), wd = round_p(bw, p);
    for (int ix = 0; ix < W; ++ix) {
        BF t1 = bf_div_si(bf_from_int(ix), W, p);   // mpfr_si_div(t1, ix, img_rw)
        BF x = bf_mul(t1, wd, p);                   // mpfr_mul(x, t1, width)
        x = bf_add(x, xm, p);                       // mpfr_add(x, x, img_xmin)
        int rc = bf_to_fixed(x, words, xs + (size_t)ix * words);
        if (rc || !fx_fits_coordinate(xs + (size_t)ix * words, words))
            return MDZGPU_ERR_RANGE;
    }
    const BF step = bf_div_si(wd, W, p);            // mpfr_div(t1, width, img_rw)
    for (int r = 0; r < nrows; ++r) {
        BF t1 = bf_mul_si(step, row0 + r, p);       // mpfr_mul_si(t1, t1, line)
        t1.sign = -t1.sign;
        BF y = bf_add(by, t1, p);                   // mpfr_sub(y, img->ymax, t1)
        int rc = bf_to_fixed(y, words, ys + (size_t)r * words);
        if (rc || !fx_fits_coordinate(ys + (size_t)r * words, words))
            return MDZGPU_ERR_RANGE;
    }
    return MDZGPU_OK;
}

int mpfr_round_to_fixed(const mdzgpu_mpval* v, long p, int words, uint32_t* out)
{
    return bf_to_fixed(round_p(bf_from_mpval(v), p), words, out);
}

}  // namespace mdz
