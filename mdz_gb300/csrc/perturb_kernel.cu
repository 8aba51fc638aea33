// Perturbation method for deep zooms.
//
// The reference has no perturbation path: its only deep-zoom method is the
// per-pixel MPFR loop (src/frac_mandel.c:25-52 and its siblings) at
// img->precision bits.  This file is the new method named for the 2^-1000
// workload, for every MDZ formula and both families:
//
// 1. Reference orbit.  Z_{k+1} = f(Z_k) + C (Z_0 = 0, Z_1 = C; Julia:
//    Z_0 = the view centre, C = the Julia constant) iterated exactly in
//    multi-limb fixed point by four warps (orbit_produce).  Numbers are L
//    signed radix-2^28 digits (value = sum d_i 2^(28 i - F), F = 28 (L-1)),
//    so every 28x28-bit product fits an IMAD.WIDE into a 64-bit column sum;
//    the columns of Re and Im are spread over the lanes and carries are
//    resolved with warp-shuffle passes.  The folds (burning ship, celtic, the
//    variant's odd steps) take their signs from the digits.  A finisher
//    rounds each Z_k to FP64 (mantissa pair + int32 exponent) and FP32 and
//    stores the exact |Z_k|^2 - 4 and, for the folded formulas, the fold
//    quantity and its exact sign.
//
// 2. Pixels.  dz = z - Z_m is kept as an FP32 mantissa pair t with an int32
//    exponent e (dz = t 2^e).  The Mandelbrot hot step is plain FP32:
//        t' = 2 Z_m t + 2^e t^2 + dc 2^-e
//    with 2^e and dc 2^-e refreshed only when |t| leaves [2^-32, 2^32].
//    FP64 is used only where precision is lost otherwise: the rebase test
//    |Z_m + dz| < |dz| (screened in FP32), the rebase itself
//    dz <- Z_m + dz, m <- 0 (Zhuoran's rebasing), the full floatexp step
//    when Z_m is tiny and dz is below the FP32 range, escape decisions
//    within 2^-14 of the bailout, and the folded formulas' steps near their
//    fold.  Pixels that lose too much precision are re-run with FP64
//    mantissas, then on the exact multi-limb kernel (perturb_run).
//
// Counts follow MDZ's convention (src/frac_mandel.c:11-20): z starts at c,
// the first update is iteration 1, the count is the first iteration whose
// result has |z|^2 > 4, or 0 if none within depth.
#include <math.h>

#include "internal.h"
#include "serve.h"

namespace mdz {
namespace {

constexpr int kTileW = 8;
constexpr int kTileH = 4;
// A pixel of the FP32 pass that steps from a reference entry at zero
// (|Z_m|^2 < 2^-120 for m past the orbit's start: the view is centred on a
// minibrot's nucleus, Z_p = 0) is handed to the FP64 pass there: around a
// nucleus the count can hinge on the position of c far below 2^-24 of its
// offset (near the edge of the minibrot's cardioid the escape time grows
// like 1/sqrt(distance)), and the FP32 steps' rounding, equivalent to
// moving c by ~2^-24 |dc| a step, then shifts it (measured on a 2^-1000
// frame centred on a period-402 nucleus: 1.1% of the pixels off by up to
// 1.5*10^5 iterations in FP32; an exact restatement of four of them needed
// ~50 significant bits).  The error estimate does not see it: the local
// dynamics are near parabolic, errors add rather than grow.  The value is
// the "bits lost" it records, above the FP32 pass's 1-bit limit.
constexpr float kFp32AtZeroLost = 64.f;
constexpr int kMaxOrbitLimbs = 80;  // F up to 2212 bits

// --------------------------------------------------------------------------
// Reference orbit
// --------------------------------------------------------------------------

__device__ __forceinline__ void digit_split(long long v, long long& digit, long long& carry)
{
    // signed digit in [-2^27, 2^27), v = digit + carry * 2^28
    digit = ((v + (1ll << 27)) & ((1ll << 28) - 1)) - (1ll << 27);
    carry = (v - digit) >> 28;
}

// value of the 4 digits below the top nonzero one as a double mantissa m and
// exponent x: value ~ m * 2^x, |m| in [0.5, 1) unless zero.  `scale` is the
// binary weight of digit 0.
__device__ void digits_to_double(const int* d, int n, int scale, double& m, int& x)
{
    int top = n - 1;
    while (top > 0 && d[top] == 0)
        --top;
    double v = (double)d[top];
    if (top >= 1)
        v += ldexp((double)d[top - 1], -28);
    if (top >= 2)
        v += ldexp((double)d[top - 2], -56);
    if (top >= 3)
        v += ldexp((double)d[top - 3], -84);
    int ex = 0;
    m = frexp(v, &ex);
    x = ex + 28 * top + scale;
    if (v == 0.0) {
        m = 0.0;
        x = 0;
    }
}

// The serial part: Z_{k+1} = Z_k^2 + C, storing the raw digits of every Z_k
// (re then im, L each) to HBM.  Two warps: warp 0 forms the columns of
// Re = Zr^2 - Zi^2 + Cr, warp 1 those of Im = 2 Zr Zi + Ci, each lane one
// column per 32-column slot; both read the packed (re, im) digit pairs from
// shared memory with 64-bit loads.  Two shuffle passes leave every digit
// within 2^27 + 2^5 of zero, small enough for the next product's 64-bit
// column sums.  Everything else about each Z_k (FP64 / FP32 roundings,
// |Z_k|^2 - 4) is done afterwards by orbit_finish_kernel, in parallel over
// k, so this loop carries only the multi-limb arithmetic.
// Progress words shared by the blocks of the fused launch.
struct OrbitProgress {
    int* raw_len;   // digit entries 0..raw_len-1 written (producer)
    int* fin_len;   // entries 0..fin_len-1 finished (finisher)
    int* done;      // producer stopped; final length in *out_len
    int* error;     // a bounded wait gave up
};

// Sign of a radix-2^28 digit vector d[0..L) whose digits are bounded well
// below 2^27 + 2^6 (the top nonzero digit decides); computed by one warp.
__device__ __forceinline__ int digits_sign_warp(const int2* z, int L, bool imag)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int s = 2; s >= 0; --s) {
        const int j = lane + 32 * s;
        const int d = j < L ? (imag ? z[j].y : z[j].x) : 0;
        const unsigned m = __ballot_sync(0xffffffffu, d != 0);
        if (m) {
            const int dt = __shfl_sync(0xffffffffu, d, 31 - __clz(m));
            return dt > 0 ? 1 : -1;
        }
    }
    return 0;
}

// The producer, run by every thread of its block (NT = blockDim.x, a
// multiple of 32, >= 64).  One step Z_k -> Z_{k+1} in two phases:
//
//  1. Products.  The L + 3 kept columns c = L-4 .. 2L-2 (3 guard columns
//     below the L digits of the result) are split into S term slices each;
//     the (column, slice) items are spread over all threads, so a thread
//     forms at most a few digit pairs (i < j = c - i, i = lo + s + S t) of
//     both parts at once: Re = sum x_i x_j - y_i y_j, Im = sum x_i y_j +
//     x_j y_i, one pair of 64-bit loads feeding four IMAD.WIDE.  Slice 0 adds
//     the square term of an even column.  Partial sums go to shared memory.
//  2. Carries.  Warp 0 (Re) and warp 1 (Im) add the S partials of their
//     columns (one column per lane and 32-column slot), apply the formula's
//     sign rules, add C, and resolve the carries in two warp-shuffle passes,
//     which leave every digit within 2^27 + 2^5 of zero, small enough for
//     the next products' 64-bit column sums; they write Z_{k+1} to shared
//     memory and its digits to HBM, and the FP32 top-digit estimate (escape
//     test) and, for burning ship, the part's sign.
//
// The column sums are exact integers, so the result does not depend on how
// the terms are sliced (any NT gives the same digits).  The escape test of
// Z_k is evaluated while Z_{k+1}'s products are formed: a step computed past
// an escape is dropped (nothing of it reaches HBM before the test).
// Everything else about each Z_k (FP64 / FP32 roundings, |Z_k|^2 - 4) is
// done afterwards by the finisher, in parallel over k.  Publishes raw_len
// every 64 steps when `prog` is given.  Inlined into each kernel that runs
// it, so that each has its own register budget.
constexpr int kOrbitMaxSlices = 8;
constexpr int kOrbitMaxCols = kMaxOrbitLimbs + 3;

struct OrbitShared {
    int2 z[kMaxOrbitLimbs];                              // Z_k digit pairs (re, im)
    int cc[2][kMaxOrbitLimbs];                           // C digits
    long long part[2][kOrbitMaxSlices][kOrbitMaxCols];   // [Re/Im][slice][column]
    float esc[2][2];   // [Re/Im][k & 1]: top two digits of Z_k as FP32
    int sgn[2][2];     // [Re/Im][k & 1]: sign of the part of Z_k (burning ship)
};

// Top-digit estimate and (burning ship) sign of one part of the Z just
// written to o.z, by the carry warp of that part (all lanes).
__device__ __forceinline__ void orbit_part_summary(OrbitShared& o, int L, int part, int slot,
                                                   bool ship)
{
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
        const int2 t1 = o.z[L - 1], t2 = o.z[L - 2];
        o.esc[part][slot] = part ? fmaf((float)t2.y, 3.7252903e-9f, (float)t1.y)
                                 : fmaf((float)t2.x, 3.7252903e-9f, (float)t1.x);
    }
    if (ship) {
        const int sg = digits_sign_warp(o.z, L, part == 1);
        if ((threadIdx.x & 31) == 0)
            o.sgn[part][slot] = sg;
    }
}

__device__ __forceinline__ void orbit_produce(const OrbitLaunch& p, const OrbitProgress* prog)
{
    __shared__ OrbitShared o;
    const int NT = blockDim.x;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int L = p.limbs;
    const int P = L + 3;           // kept columns cbase .. cbase + P - 1
    const int cbase = L - 4;       // lowest column computed (3 guard columns)
    const int nslots = (P + 31) / 32;
    int S = NT / P;
    S = S < 1 ? 1 : (S > kOrbitMaxSlices ? kOrbitMaxSlices : S);
    const bool from_z0 = p.z0_re != nullptr;   // Julia: Z_0 given, k starts at 0
    const bool ship = p.fractal == MDZ_BURNING_SHIP;
    const bool celtic = p.fractal == MDZ_GENERALIZED_CELTIC;
    const bool variant = p.fractal == MDZ_VARIANT;
    for (int j = threadIdx.x; j < L; j += NT) {
        o.cc[0][j] = p.c_re[j];
        o.cc[1][j] = p.c_im[j];
        if (from_z0) {
            o.z[j] = make_int2(p.z0_re[j], p.z0_im[j]);
            p.digits[j] = p.z0_re[j];
            p.digits[L + j] = p.z0_im[j];
        } else {
            o.z[j] = make_int2(p.c_re[j], p.c_im[j]);
            p.digits[j] = 0;                    // Z_0 = 0
            p.digits[L + j] = 0;
            p.digits[2 * L + j] = p.c_re[j];    // Z_1 = C
            p.digits[3 * L + j] = p.c_im[j];
        }
    }
    __threadfence();
    __syncthreads();
    int k = from_z0 ? 0 : 1;
    if (warp < 2)
        orbit_part_summary(o, L, warp, k & 1, ship);
    for (;; ++k) {
        __syncthreads();  // A: Z_k, its estimate and signs complete
        if (prog && (k & 63) == 0 && threadIdx.x == 0)
            *(volatile int*)prog->raw_len = k + 1;
        // phase 1: partial column sums of Z_k^2
        for (int q = threadIdx.x; q < S * P; q += NT) {
            const int s = q / P;
            const int pos = q - s * P;
            const int c = cbase + pos;
            const int lo = c - (L - 1) > 0 ? c - (L - 1) : 0;
            const int hi = (c - 1) >> 1;  // last i with i < j = c - i
            long long r0 = 0, r1 = 0, m0 = 0, m1 = 0;
            int i = lo + s;
            for (; i + S <= hi; i += 2 * S) {
                const int2 a = o.z[i], b = o.z[c - i];
                const int2 a2 = o.z[i + S], b2 = o.z[c - i - S];
                r0 += (long long)a.x * b.x - (long long)a.y * b.y;
                m0 += (long long)a.x * b.y + (long long)b.x * a.y;
                r1 += (long long)a2.x * b2.x - (long long)a2.y * b2.y;
                m1 += (long long)a2.x * b2.y + (long long)b2.x * a2.y;
            }
            if (i <= hi) {
                const int2 a = o.z[i], b = o.z[c - i];
                r0 += (long long)a.x * b.x - (long long)a.y * b.y;
                m0 += (long long)a.x * b.y + (long long)b.x * a.y;
            }
            long long re = 2 * (r0 + r1), im = 2 * (m0 + m1);
            if (s == 0 && !(c & 1)) {
                const int2 h = o.z[c >> 1];
                re += (long long)h.x * h.x - (long long)h.y * h.y;
                im += 2 * (long long)h.x * h.y;
            }
            o.part[0][s][pos] = re;
            o.part[1][s][pos] = im;
        }
        const float ea = o.esc[0][k & 1], eb = o.esc[1][k & 1];
        const bool stop = fmaf(ea, ea, eb * eb) > 4.0f || k >= p.max_k;
        const int sxy = ship ? o.sgn[0][k & 1] * o.sgn[1][k & 1] : 1;
        __syncthreads();  // B: partial sums in place; every read of Z_k done
        if (stop)
            break;
        if (warp >= 2)
            continue;
        // phase 2 (warp 0: Re, warp 1: Im): Z_{k+1}
        const int part = warp;
        // celtic fold of this step (every step, or the variant's odd ones)
        const bool fold_re = part == 0 && (celtic || (variant && (k & 1) == p.fold_parity));
        long long v[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int pos = lane + 32 * t;
            long long acc = 0;
            if (t < nslots && pos < P) {
                for (int s = 0; s < S; ++s)
                    acc += o.part[part][s][pos];
                // burning ship: Im' = 2 |Re| |Im| + Ci = sign(Re) sign(Im) 2 Re Im + Ci
                if (part == 1)
                    acc *= sxy;
                // celtic adds Cr after the fold (below)
                if (pos >= 3 && !fold_re)
                    acc += o.cc[part][pos - 3];
            }
            v[t] = acc;
        }
        // carry propagation: column pos+1 is lane+1 (slot t) or lane 0 of
        // slot t+1; two passes bound every digit by 2^27 + 2^5
        auto carry2 = [&]() {
#pragma unroll
            for (int pass = 0; pass < 2; ++pass) {
                long long dg[3], cy[3];
#pragma unroll
                for (int t = 0; t < 3; ++t)
                    digit_split(v[t], dg[t], cy[t]);
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    if (t >= nslots)
                        break;
                    long long in = __shfl_up_sync(0xffffffffu, cy[t], 1);
                    const long long wrap =
                        __shfl_sync(0xffffffffu, t > 0 ? cy[t - 1] : 0ll, 31);
                    if (lane == 0)
                        in = wrap;
                    v[t] = dg[t] + in;
                }
            }
        };
        carry2();
        if (fold_re) {
            // Re' = |Re^2 - Im^2| + Cr: the sign of the carried digits is
            // that of their most significant nonzero one
            int sg = 0;
#pragma unroll
            for (int t = 2; t >= 0; --t) {
                const int pos = lane + 32 * t;
                const bool ok = t < nslots && pos < P && v[t] != 0;
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (m && !sg) {
                    const long long x = __shfl_sync(0xffffffffu, v[t], 31 - __clz(m));
                    sg = x > 0 ? 1 : -1;
                }
            }
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const int pos = lane + 32 * t;
                if (sg < 0)
                    v[t] = -v[t];
                if (t < nslots && pos < P && pos >= 3)
                    v[t] += o.cc[0][pos - 3];
            }
            carry2();
        }
        int* out = p.digits + (size_t)(k + 1) * 2 * L + part * L;
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int pos = lane + 32 * t;
            if (t < nslots && pos < P && pos >= 3) {
                const int d = (int)v[t];
                if (part == 0)
                    o.z[pos - 3].x = d;
                else
                    o.z[pos - 3].y = d;
                out[pos - 3] = d;
            }
        }
        orbit_part_summary(o, L, part, (k + 1) & 1, ship);
        if (prog && ((k + 1) & 63) == 0)
            __threadfence();  // Z_{k+1}'s digits before raw_len = k + 2
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        *p.out_len = k + 1;  // entries 0..k are valid
        if (prog) {
            *(volatile int*)prog->raw_len = k + 1;
            __threadfence();
            *(volatile int*)prog->done = 1;
        }
    }
}

// The producer of the standalone orbit kernels (orbit_kernel,
// orbit_stream_kernel), with every thread's work fixed before the loop.
// Same column sums and carries as orbit_produce, so the same digits; laid
// out for the shortest serial step: the kept columns are split into
// kOrbitLeanSlices term slices, and thread q < slices x columns owns one
// (slice, column) item whose at most MAXP digit pairs are known before the
// first step (shared-memory indices, padded with a zero entry, so every
// thread runs the same straight-line code); warps 0 and 1 then add the
// slices' partial sums of their columns (NSLOT per lane), add C, fold and
// resolve the carries as orbit_produce does.  The generic loop spent most
// of its serial step on per-step index arithmetic (divisions, variable trip
// counts); orbit_produce stays for the fused launch, whose blocks are
// smaller than slices x columns.
constexpr int kOrbitLeanSlices = 8;

template <int MAXP, int NSLOT>
__device__ __forceinline__ void orbit_produce_lean(const OrbitLaunch& p, const OrbitProgress* prog)
{
    constexpr int S = kOrbitLeanSlices;
    __shared__ int2 z[kMaxOrbitLimbs + 1];                  // z[L] stays zero
    __shared__ int cc[2][kMaxOrbitLimbs];
    __shared__ long long part[2][S][kMaxOrbitLimbs + 3];
    __shared__ float esc[2][2];
    __shared__ int sgn[2][2];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int L = p.limbs;
    const int P = L + 3;
    const int cbase = L - 4;
    const bool from_z0 = p.z0_re != nullptr;
    const bool ship = p.fractal == MDZ_BURNING_SHIP;
    const bool celtic = p.fractal == MDZ_GENERALIZED_CELTIC;
    const bool variant = p.fractal == MDZ_VARIANT;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        cc[0][j] = p.c_re[j];
        cc[1][j] = p.c_im[j];
        if (from_z0) {
            z[j] = make_int2(p.z0_re[j], p.z0_im[j]);
            p.digits[j] = p.z0_re[j];
            p.digits[L + j] = p.z0_im[j];
        } else {
            z[j] = make_int2(p.c_re[j], p.c_im[j]);
            p.digits[j] = 0;                    // Z_0 = 0
            p.digits[L + j] = 0;
            p.digits[2 * L + j] = p.c_re[j];    // Z_1 = C
            p.digits[3 * L + j] = p.c_im[j];
        }
    }
    if (threadIdx.x == 0)
        z[L] = make_int2(0, 0);
    // this thread's item and its pair indices
    const int q = threadIdx.x;
    const bool worker = q < S * P;
    const int s = worker ? q / P : 0;
    const int pos = worker ? q - s * P : 0;
    const int c = cbase + pos;
    const int lo = c - (L - 1) > 0 ? c - (L - 1) : 0;
    const int hi = (c - 1) >> 1;
    int ia[MAXP], ib[MAXP];
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
        const int i = lo + s + S * j;
        const bool ok = worker && i <= hi;
        ia[j] = ok ? i : L;
        ib[j] = ok ? c - i : L;
    }
    const int ih = (worker && s == 0 && !(c & 1)) ? (c >> 1) : L;
    __threadfence();
    __syncthreads();
    int k = from_z0 ? 0 : 1;
    // top-digit estimate (escape test) and, for burning ship, the sign of
    // part pt of the Z just written (all lanes of warp pt)
    auto summary = [&](int pt, int slot) {
        __syncwarp();
        if (lane == 0) {
            const int2 t1 = z[L - 1], t2 = z[L - 2];
            esc[pt][slot] = pt ? fmaf((float)t2.y, 3.7252903e-9f, (float)t1.y)
                               : fmaf((float)t2.x, 3.7252903e-9f, (float)t1.x);
        }
        if (ship) {
            const int sg = digits_sign_warp(z, L, pt == 1);
            if (lane == 0)
                sgn[pt][slot] = sg;
        }
    };
    if (warp < 2)
        summary(warp, k & 1);
    for (;; ++k) {
        __syncthreads();  // A: Z_k, its estimate and signs complete
        if (prog && (k & 63) == 0 && threadIdx.x == 0)
            *(volatile int*)prog->raw_len = k + 1;
        if (worker) {
            long long r0 = 0, r1 = 0, m0 = 0, m1 = 0;
#pragma unroll
            for (int j = 0; j < MAXP; ++j) {
                const int2 a = z[ia[j]], b = z[ib[j]];
                if (j & 1) {
                    r1 += (long long)a.x * b.x;
                    r1 -= (long long)a.y * b.y;
                    m1 += (long long)a.x * b.y;
                    m1 += (long long)b.x * a.y;
                } else {
                    r0 += (long long)a.x * b.x;
                    r0 -= (long long)a.y * b.y;
                    m0 += (long long)a.x * b.y;
                    m0 += (long long)b.x * a.y;
                }
            }
            const int2 h = z[ih];
            long long re = 2 * (r0 + r1), im = 2 * (m0 + m1);
            re += (long long)h.x * h.x;
            re -= (long long)h.y * h.y;
            im += 2 * ((long long)h.x * h.y);
            part[0][s][pos] = re;
            part[1][s][pos] = im;
        }
        const float ea = esc[0][k & 1], eb = esc[1][k & 1];
        const bool stop = fmaf(ea, ea, eb * eb) > 4.0f || k >= p.max_k;
        const int sxy = ship ? sgn[0][k & 1] * sgn[1][k & 1] : 1;
        __syncthreads();  // B: partial sums in place; every read of Z_k done
        if (stop)
            break;
        if (warp >= 2)
            continue;
        // Z_{k+1}: warp 0 the real part, warp 1 the imaginary part
        const int pt = warp;
        const bool fold_re = pt == 0 && (celtic || (variant && (k & 1) == p.fold_parity));
        long long v[NSLOT];
#pragma unroll
        for (int t = 0; t < NSLOT; ++t) {
            const int pp = lane + 32 * t;
            long long a = 0;
            if (pp < P) {
                long long u[S];
#pragma unroll
                for (int ss = 0; ss < S; ++ss)
                    u[ss] = part[pt][ss][pp];
                a = ((u[0] + u[1]) + (u[2] + u[3])) + ((u[4] + u[5]) + (u[6] + u[7]));
                if (pt == 1)
                    a *= sxy;
                if (pp >= 3 && !fold_re)
                    a += cc[pt][pp - 3];
            }
            v[t] = a;
        }
        auto carry2 = [&]() {
#pragma unroll
            for (int pass = 0; pass < 2; ++pass) {
                long long dg[NSLOT], cy[NSLOT];
#pragma unroll
                for (int t = 0; t < NSLOT; ++t)
                    digit_split(v[t], dg[t], cy[t]);
#pragma unroll
                for (int t = 0; t < NSLOT; ++t) {
                    long long in = __shfl_up_sync(0xffffffffu, cy[t], 1);
                    const long long wrap =
                        __shfl_sync(0xffffffffu, t > 0 ? cy[t - 1] : 0ll, 31);
                    if (lane == 0)
                        in = wrap;
                    v[t] = dg[t] + in;
                }
            }
        };
        carry2();
        if (fold_re) {
            int sg = 0;
#pragma unroll
            for (int t = NSLOT - 1; t >= 0; --t) {
                const int pp = lane + 32 * t;
                const bool ok = pp < P && v[t] != 0;
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (m && !sg) {
                    const long long x = __shfl_sync(0xffffffffu, v[t], 31 - __clz(m));
                    sg = x > 0 ? 1 : -1;
                }
            }
#pragma unroll
            for (int t = 0; t < NSLOT; ++t) {
                const int pp = lane + 32 * t;
                if (sg < 0)
                    v[t] = -v[t];
                if (pp < P && pp >= 3)
                    v[t] += cc[0][pp - 3];
            }
            carry2();
        }
        int* out = p.digits + (size_t)(k + 1) * 2 * L + pt * L;
#pragma unroll
        for (int t = 0; t < NSLOT; ++t) {
            const int pp = lane + 32 * t;
            if (pp >= 3 && pp < P) {
                const int d = (int)v[t];
                if (pt == 0)
                    z[pp - 3].x = d;
                else
                    z[pp - 3].y = d;
                out[pp - 3] = d;
            }
        }
        summary(pt, (k + 1) & 1);
        if (prog && ((k + 1) & 63) == 0)
            __threadfence();  // Z_{k+1}'s digits before raw_len = k + 2
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        *p.out_len = k + 1;  // entries 0..k are valid
        if (prog) {
            *(volatile int*)prog->raw_len = k + 1;
            __threadfence();
            *(volatile int*)prog->done = 1;
        }
    }
}

// (MAXP, NSLOT) of the lean producer for L digits: a column holds at most
// floor(L / 2) pairs, spread over 8 slices; L + 3 columns over 32 lanes.
#define MDZ_ORBIT_LEAN_CASES(X) \
    X(17, 1, 1) X(29, 2, 1) X(33, 2, 2) X(49, 3, 2) X(61, 4, 2) X(65, 4, 3) X(80, 5, 3)

// Threads of a lean launch: slices x columns, rounded to 512 or 1024 (the
// finisher of the streamed orbit works in batches of its block size, which
// must divide 1024).
__host__ __device__ constexpr int orbit_lean_threads(int L)
{
    return kOrbitLeanSlices * (L + 3) <= 512 ? 512 : 1024;
}

template <int MAXP, int NSLOT>
__global__ void __launch_bounds__(1024) orbit_kernel_lean(OrbitLaunch p)
{
    unsigned smid = 0;
    if (p.sm_busy) {
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        smid %= (unsigned)p.sm_words;
        if (threadIdx.x == 0)
            atomicAdd(p.sm_busy + smid, 1);
    }
    orbit_produce_lean<MAXP, NSLOT>(p, nullptr);
    if (p.sm_busy && threadIdx.x == 0)
        atomicSub(p.sm_busy + smid, 1);
}

// Per entry k (one thread each): the FP64 pair with its exponent, the FP32
// pair, and D_k = |Z_k|^2 - 4 -- from FP64 when that is far from 0,
// otherwise exactly from the digits (the full 2L-column sum of squares),
// because the escape test of a pixel with a tiny dz needs the sign of
// D_k + 2 Re(conj(Z_k) dz) + |dz|^2 and FP32 / FP64 roundings of Z_k can
// not give it when |Z_k| is within 2^-20 of 2.
__device__ __noinline__ void finish_entry(const OrbitLaunch& p, int k, bool from_l2)
{
    const int L = p.limbs;
    int dr[kMaxOrbitLimbs], di[kMaxOrbitLimbs];
    const int* src = p.digits + (size_t)k * 2 * L;
    for (int j = 0; j < L; ++j) {
        // in the fused launch the digits were written by another block while
        // this one runs: read them from L2, never from a stale L1 line
        dr[j] = from_l2 ? __ldcg(src + j) : src[j];
        di[j] = from_l2 ? __ldcg(src + L + j) : src[L + j];
    }
    const int F = 28 * (L - 1);
    double mr, mi;
    int xr, xi;
    digits_to_double(dr, L, -F, mr, xr);
    digits_to_double(di, L, -F, mi, xi);
    const int xe = (mr == 0.0) ? xi : (mi == 0.0 ? xr : max(xr, xi));
    const double nr = ldexp(mr, xr - xe), ni = ldexp(mi, xi - xe);
    const double vr = ldexp(nr, xe), vi = ldexp(ni, xe);
    if (xe < -960) {
        p.zd[k] = make_double2(nr, ni);
        p.ze[k] = xe;
    } else {
        p.zd[k] = make_double2(vr, vi);
        p.ze[k] = 0;
    }
    const float fx = (float)vr, fy = (float)vi;
    // burning ship / celtic: the fold quantity F_k and its exact sign
    float fold_sign = 1.f;
    if (p.fractal == MDZ_BURNING_SHIP || p.fractal == MDZ_GENERALIZED_CELTIC
        || p.fractal == MDZ_VARIANT) {
        double fmv;
        int fev;
        if (p.fractal == MDZ_BURNING_SHIP) {
            // F = Re Im: the product of the two 53-bit roundings
            fmv = mr * mi;
            fev = xr + xi;
        } else {
            // F = Re^2 - Im^2 = (|Re| - |Im|)(|Re| + |Im|), the difference
            // formed exactly on the digits
            const int sr = mr < 0.0 ? -1 : 1, si = mi < 0.0 ? -1 : 1;
            int dd[kMaxOrbitLimbs], ss[kMaxOrbitLimbs];
            long long cd = 0, cs = 0;
            for (int j = 0; j < L; ++j) {
                long long d, cy;
                digit_split(sr * (long long)dr[j] - si * (long long)di[j] + cd, d, cy);
                dd[j] = (int)d;
                cd = cy;
                digit_split(sr * (long long)dr[j] + si * (long long)di[j] + cs, d, cy);
                ss[j] = (int)d;
                cs = cy;
            }
            // |values| < 8: the last carries stay within the top digit
            dd[L - 1] += (int)(cd << 28);
            ss[L - 1] += (int)(cs << 28);
            double md, ms;
            int xd, xs;
            digits_to_double(dd, L, -F, md, xd);
            digits_to_double(ss, L, -F, ms, xs);
            fmv = md * ms;
            fev = xd + xs;
        }
        if (fmv < 0.0)
            fold_sign = -1.f;
        if (p.fm) {
            p.fm[k] = fmv;
            p.fe[k] = fmv == 0.0 ? -100000 : fev;
        }
    }
    // 2 Z_k (the step multiplies by it; doubling is exact) and |Z_k|^2
    // exactly as the pixel loop forms |z|^2 when dz vanishes in FP32
    p.zq[k] = make_float4(fx + fx, fy + fy, fmaf(fx, fx, fy * fy), fold_sign);
    const double d_approx = vr * vr + vi * vi - 4.0;
    if (fabs(d_approx) > 9.5367431640625e-7 /* 2^-20 */) {
        p.dd[k] = d_approx;
        p.de[k] = 0;
        return;
    }
    // exact: columns of Zr^2 + Zi^2 (weight of column c: 2^(28 c - 2F)),
    // minus 4 in the top column, carries resolved serially
    long long col[2 * kMaxOrbitLimbs];
    int dig[2 * kMaxOrbitLimbs];
    const int ncol = 2 * L - 1;
    for (int c = 0; c < ncol; ++c) {
        long long acc = 0;
        const int ilo = c - (L - 1) > 0 ? c - (L - 1) : 0;
        const int ihi = c < L - 1 ? c : L - 1;
        for (int i = ilo; i <= ihi; ++i)
            acc += (long long)dr[i] * dr[c - i] + (long long)di[i] * di[c - i];
        col[c] = acc;
    }
    col[ncol - 1] -= 4;
    long long carry = 0;
    for (int c = 0; c < ncol; ++c) {
        long long v = col[c] + carry, d, cy;
        digit_split(v, d, cy);
        dig[c] = (int)d;
        carry = cy;
    }
    // anything left in `carry` is a multiple of 2^(28 ncol - 2F) = 2^28
    // above the top column: fold it back in (|D| < 1 here, so it is 0 or a
    // single unit that cancels the top digit)
    dig[ncol - 1] += (int)(carry << 28);
    double m;
    int x;
    digits_to_double(dig, ncol, -2 * F, m, x);
    p.dd[k] = m;
    p.de[k] = x;
}

// Bit k of p.tiny: |Z_k|^2 < 2^-120 in FP32 (the pixel pass takes the full
// floatexp step there when dz is below the FP32 range); bit k of p.att:
// |Z_k|^2 in the FP32 escape band or below the rebase screen's 2^-60 (a
// superset of tiny: the deep-zoom blocks skip their tests where it is
// clear); bit k of p.axis:
// |F_k| < 2^-99 (burning ship / celtic: a dz of the FP32 range can carry a
// pixel across the fold there).  Written per warp of 32 consecutive
// entries, so every word has one writer.
__device__ __forceinline__ void write_tiny_bits(const OrbitLaunch& p, int k, bool valid)
{
    bool tiny = false, axis = false, att = false;
    if (valid) {
        const float m2 = p.zq[k].z;
        tiny = m2 < 7.5e-37f;
        // as the FP32 pixel loop tests |z|^2 = |Z_k|^2 (Mant<float>)
        att = m2 > 4.0f - 6.1035156e-5f || m2 < 8.7e-19f;
        if (p.fm)
            axis = p.fm[k] == 0.0 || p.fe[k] <= -99;
    }
    const unsigned bits = __ballot_sync(0xffffffffu, tiny);
    const unsigned abits = __ballot_sync(0xffffffffu, axis);
    const unsigned tbits = __ballot_sync(0xffffffffu, att);
    if ((threadIdx.x & 31) == 0 && k >= 0) {
        if (p.tiny)
            p.tiny[k >> 5] = bits;
        if (p.axis)
            p.axis[k >> 5] = abits;
        if (p.att)
            p.att[k >> 5] = tbits;
    }
}

__global__ void __launch_bounds__(128) orbit_finish_kernel(OrbitLaunch p)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = k < *p.out_len;
    if (valid)
        finish_entry(p, k, false);
    write_tiny_bits(p, k, valid);
}

// The finisher of the streamed orbit (one block of B = blockDim.x threads, a
// multiple of 32 dividing 1024): finishes the orbit in batches of B entries
// as the producer publishes them and publishes fin_len in units of 1024
// entries, so a consumer never reads a cache line holding an unfinished
// entry.
__device__ void orbit_finisher(const OrbitLaunch& p, const OrbitProgress& g)
{
    __shared__ int s_avail, s_done, s_err;
    int fin = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            int spins = 0, r = 0, d = 0, err = 0;
            for (;;) {
                d = *(volatile int*)g.done;
                r = d ? *(volatile int*)p.out_len : *(volatile int*)g.raw_len;
                if (d || r >= fin + (int)blockDim.x)
                    break;
                if (*(volatile int*)g.error || ++spins > p.spin_limit) {
                    err = 1;
                    break;
                }
                __nanosleep(256);
            }
            s_avail = r;
            s_done = d;
            s_err = err;
        }
        __syncthreads();
        const int avail = s_avail, dn = s_done;
        if (s_err) {
            if (threadIdx.x == 0)
                atomicExch(g.error, 1);
            return;
        }
        const int end = min(avail, fin + (int)blockDim.x);
        const int k = fin + (int)threadIdx.x;
        if (k < end)
            finish_entry(p, k, true);
        write_tiny_bits(p, k, k < end);
        __threadfence();
        __syncthreads();
        // publish in whole 1024-entry units (one 128-byte line of the tiny
        // mask, 128 lines of zq) or at the end, so that no cache line a
        // consumer reads holds an entry that is not finished yet
        if (threadIdx.x == 0 && ((end & 1023) == 0 || (dn && end >= avail)))
            *(volatile int*)g.fin_len = end;
        fin = end;
        if (dn && fin >= avail)
            return;
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// Pixels
// --------------------------------------------------------------------------

// Mantissa traits of the pixel loop: FP32 (the fast pass) or FP64 (the
// escalation pass for pixels whose rebases cancelled too many bits).
template <class T>
struct Mant;
template <>
struct Mant<float> {
    static constexpr int kMinExp = -149;     // below: 2^e is 0
    static constexpr int kSlowExp = -120;    // dz^2 term may vanish below
    static constexpr int kSqExp = -63;       // 2^(2e) representable above
    static constexpr float kTinyZ2 = 7.5e-37f;   // |Z|^2 < 2^-120
    static constexpr float kGlitchZ2 = 8.7e-19f; // |Z|^2 < 2^-60
    static constexpr int kForceSlow = 120;   // dc 2^-e would overflow above
    static constexpr float kFoldEps = 9.5367431640625e-7f;  // 2^-20: sign margin
    static constexpr double kEps2x16 = 5.684341886080802e-14;  // 16 (2^-24)^2
    __device__ static float scale(float x, int e) { return ldexpf(x, e); }
    __device__ static float fma_(float a, float b, float c) { return fmaf(a, b, c); }
    __device__ static int exponent_of(float a) { return ((__float_as_int(a) >> 23) & 0xff) - 127; }
};
template <>
struct Mant<double> {
    static constexpr int kMinExp = -1074;
    static constexpr int kSlowExp = -1000;
    static constexpr int kSqExp = -511;
    static constexpr double kTinyZ2 = 1e-300;
    static constexpr double kGlitchZ2 = 8.7e-19;
    static constexpr int kForceSlow = 1000;
    static constexpr double kFoldEps = 3.552713678800501e-15;  // 2^-48
    static constexpr double kEps2x16 = 1.9721522630525295e-31;  // 16 (2^-53)^2
    __device__ static double scale(double x, int e) { return ldexp(x, e); }
    __device__ static double fma_(double a, double b, double c) { return fma(a, b, c); }
    __device__ static int exponent_of(double a) { return ilogb(a); }
};

template <class T>
struct PixState {
    T tr, ti;       // dz mantissas
    int e;          // dz = t * 2^e
    T s;            // 2^e (0 below the range)
    T s2scr;        // (1 + 2^-16) 2^(2e): the rebase screen; 0 when 2^(2e) underflows
    T dcr, dci;     // dc * 2^-e
    bool careful;   // slow_if_tiny || force_slow
    bool slow_if_tiny;
    bool force_slow;
    // folded formulas: estimate of the absolute error of z accumulated by
    // the rounding of the deltas, err^2 = ke e2 2^(2e) (see fold_ke)
    T e2;
    T ke;
    T kb;           // 2^18 ke 2^(2e): e2 kb = (2^9 err)^2; 0 when 2^(2e) underflows
    T sm;           // 2^-5 2^e: the fold margin per unit of |t|
};

template <class T>
__device__ __forceinline__ void refresh_scale(PixState<T>& st, T dcm_r, T dcm_i, int dce)
{
    st.s = Mant<T>::scale((T)1, st.e);
    st.s2scr = st.e >= Mant<T>::kSqExp ? (T)1.0000152587890625 * st.s * st.s : (T)0;
    st.dcr = Mant<T>::scale(dcm_r, dce - st.e);
    st.dci = Mant<T>::scale(dcm_i, dce - st.e);
    st.slow_if_tiny = st.e < Mant<T>::kSlowExp;
    // dc * 2^-e would overflow (dz far below dc); a pixel with dc == 0
    // is the reference point itself and never needs it.
    st.force_slow = (dcm_r != (T)0 || dcm_i != (T)0) && (dce - st.e) > Mant<T>::kForceSlow;
    st.careful = st.slow_if_tiny || st.force_slow;
    st.kb = st.e >= Mant<T>::kSqExp ? (T)262144 * st.ke * st.s * st.s : (T)0;
    st.sm = (T)0.03125 * st.s;
}

// Set t, e from a double pair scaled by 2^E.
template <class T>
__device__ __forceinline__ void set_from_double(PixState<T>& st, double xr, double xi, int E)
{
    const double a = fmax(fabs(xr), fabs(xi));
    if (a == 0.0) {
        st.tr = (T)0;
        st.ti = (T)0;
        st.e = E;
        return;
    }
    const int k = ilogb(a);
    st.tr = (T)ldexp(xr, -k);
    st.ti = (T)ldexp(xi, -k);
    st.e = E + k;
}

__device__ __forceinline__ int dexp_of(double x)
{
    return x == 0.0 ? -100000 : ilogb(x);
}

// ---- rare paths, kept out of the hot loop's instruction stream ----

// dz <- Z_m + dz, m <- 0 (Zhuoran's rebase; at the end of the orbit, or when
// |Z_m + dz| < |dz|).  Adds the bits the sum cancelled to `lost`.  When
// `only_if_glitch`, rebases only if |Z_m + dz| < |dz| and returns whether it
// did.
template <class T>
__device__ __forceinline__ bool rebase_fp64(const PerturbLaunch& p, int m, PixState<T>& st,
                                         T dcf_r, T dcf_i, int dce, float& lost,
                                         bool only_if_glitch)
{
    const double2 zd = p.zd[m];
    const int ze = p.ze[m];
    const int E = max(dexp_of(fmax(fabs(zd.x), fabs(zd.y))) + ze, st.e + 40);
    const double dr = ldexp((double)st.tr, st.e - E), di = ldexp((double)st.ti, st.e - E);
    const double fr = ldexp(zd.x, ze - E) + dr, fi = ldexp(zd.y, ze - E) + di;
    const double z2 = fr * fr + fi * fi, d2 = dr * dr + di * di;
    if (only_if_glitch && !(z2 < d2))
        return false;
    if (d2 > z2 && z2 > 0.0)
        lost += 0.5f * (float)log2(d2 / z2);
    set_from_double(st, fr, fi, E);
    refresh_scale(st, dcf_r, dcf_i, dce);
    return true;
}

// full floatexp step in FP64: dz' = 2 Z dz + dz^2 + dc
template <class T>
__device__ __forceinline__ void slow_step(const PerturbLaunch& p, int m, PixState<T>& st, T dcf_r,
                                       T dcf_i, double dcm_r, double dcm_i, int dce)
{
    const double2 zd = p.zd[m];
    const int ze = p.ze[m];
    const double tr = (double)st.tr, ti = (double)st.ti;
    const double ar = 2.0 * (zd.x * tr - zd.y * ti), ai = 2.0 * (zd.x * ti + zd.y * tr);
    const int ae = ze + st.e;
    const double br = tr * tr - ti * ti, bi = 2.0 * tr * ti;
    const int be = 2 * st.e;
    const int E = max(max(dexp_of(fmax(fabs(ar), fabs(ai))) + ae,
                          dexp_of(fmax(fabs(br), fabs(bi))) + be),
                      dexp_of(fmax(fabs(dcm_r), fabs(dcm_i))) + dce);
    const double rr = ldexp(ar, ae - E) + ldexp(br, be - E) + ldexp(dcm_r, dce - E);
    const double ri = ldexp(ai, ae - E) + ldexp(bi, be - E) + ldexp(dcm_i, dce - E);
    set_from_double(st, rr, ri, E);
    refresh_scale(st, dcf_r, dcf_i, dce);
}

// |z|^2 > 4 decided from D_m = |Z_m|^2 - 4 (exact, from the orbit digits):
// |z|^2 - 4 = D_m + 2 Re(conj(Z_m) dz) + |dz|^2, in FP64 with exponents.
// (Handing the decisions that fall within the deltas' own rounding error to
// the FP64 pass was measured: on the 2^-1000 frame it sent ~0.2% of the
// pixels -- those near the isoline its centre sits on -- through the FP64
// and multi-limb passes at depth 200000, +230 ms a frame, for no change in
// the 4096 scored samples; the decision stays here.)
template <class T>
__device__ __forceinline__ bool escape_exact(const PerturbLaunch& p, int m, const PixState<T>& st)
{
    const double2 zd = p.zd[m];
    const int ze = p.ze[m];
    const double dd = p.dd[m];
    const int de = p.de[m];
    const double t2 = 2.0 * (zd.x * (double)st.tr + zd.y * (double)st.ti);
    const int e2 = ze + st.e;
    const double t3 = (double)st.tr * st.tr + (double)st.ti * st.ti;
    const int e3 = 2 * st.e;
    const int E = max(max(dexp_of(dd) + de, dexp_of(t2) + e2), dexp_of(t3) + e3);
    const double v = ldexp(dd, de - E) + ldexp(t2, e2 - E) + ldexp(t3, e3 - E);
    return v > 0.0;
}

// |Z_m|^2 below the FP32 range of the dz^2 term (the slow-step trigger):
// FP32 reads the orbit's bit mask, FP64 tests the value itself.
template <class T>
__device__ __forceinline__ bool z_tiny(const PerturbLaunch& p, int m, T zx, T zy)
{
    if (sizeof(T) == 4)
        return (__ldg(p.tiny + (m >> 5)) >> (m & 31)) & 1u;
    return zx * zx + zy * zy < (T)Mant<T>::kTinyZ2;
}

// five_clear: bits m .. m+4 of a bit mask are all clear (the attention mask
// of the deep-zoom blocks).
// four_not_tiny: none of Z_m .. Z_{m+3} is tiny (FP32 bit mask).  The next word
// is read only when bits m .. m+3 reach into it: a word holding no entry
// below the orbit progress must not be loaded (the finisher publishes whole
// 128-byte lines of the mask, and a line loaded early would stay stale in
// this SM's L1 for the rest of the launch).
__device__ __forceinline__ bool five_clear(const unsigned* mask, int m)
{
    const unsigned lo = __ldg(mask + (m >> 5));
    const unsigned hi = ((unsigned)m & 31u) > 27u ? __ldg(mask + (m >> 5) + 1) : 0u;
    return (__funnelshift_r(lo, hi, (unsigned)m & 31u) & 0x1fu) == 0u;
}

__device__ __forceinline__ bool four_not_tiny(const PerturbLaunch& p, int m)
{
    const unsigned lo = __ldg(p.tiny + (m >> 5));
    const unsigned hi = ((unsigned)m & 31u) > 28u ? __ldg(p.tiny + (m >> 5) + 1) : 0u;
    return (__funnelshift_r(lo, hi, (unsigned)m & 31u) & 0xfu) == 0u;
}

template <class T>
__device__ __forceinline__ void load_z(const PerturbLaunch& p, int m, T& zx, T& zy)
{
    if (sizeof(T) == 4) {
        const float4 z = p.zq[m];   // holds 2 Z_m (exact)
        zx = (T)(0.5f * z.x);
        zy = (T)(0.5f * z.y);
    } else {
        const double2 zd = p.zd[m];
        const int ze = p.ze[m];
        zx = (T)(ze ? ldexp(zd.x, ze) : zd.x);
        zy = (T)(ze ? ldexp(zd.y, ze) : zd.y);
    }
}

// Fold sign of entry m (burning ship: sign(Re Im), celtic: sign(Re^2 - Im^2),
// exact from the orbit digits; +1 at 0).
__device__ __forceinline__ float fold_sign(const PerturbLaunch& p, int m)
{
    return p.zq[m].w;
}

__device__ __forceinline__ bool axis_bit(const PerturbLaunch& p, int m)
{
    return (__ldg(p.axis + (m >> 5)) >> (m & 31)) & 1u;
}

__device__ __forceinline__ bool four_not_axis(const PerturbLaunch& p, int m)
{
    const unsigned lo = __ldg(p.axis + (m >> 5));
    const unsigned hi = ((unsigned)m & 31u) > 28u ? __ldg(p.axis + (m >> 5) + 1) : 0u;
    return (__funnelshift_r(lo, hi, (unsigned)m & 31u) & 0xfu) == 0u;
}

// The current z = Z_m + dz is on the same side of the fold as Z_m, and the
// T-rounded values say so with a margin (burning ship: both signs of z
// agree with those of Z_m's product; celtic: |Re z| - |Im z| has the sign of
// Re Z^2 - Im Z^2).  The margin covers the rounding of z (eps) and the
// error of dz: `dzm` = 2^-5 |dz|, well above the relative error estimate
// the pixel loop enforces (2^-8).
template <class T, int FR>
__device__ __forceinline__ bool fold_certain(T zr, T zi, T Zx, T Zy, T fs, T dzm)
{
    const T eps = (T)Mant<T>::kFoldEps;
    if (FR == MDZ_BURNING_SHIP) {
        const bool neg = (zr < (T)0) != (zi < (T)0);
        return (neg ? (T)-1 : (T)1) == fs && fabs(zr) > fmax(eps * fabs(Zx), dzm)
               && fabs(zi) > fmax(eps * fabs(Zy), dzm);
    }
    const T ar = fabs(zr), ai = fabs(zi);
    return fs * (ar - ai) > Mant<T>::fma_(eps, ar + ai, dzm + dzm);
}

// Error estimate of the folded formulas' deltas.  Every step rounds t
// (inj <= 4 eps |t'|), and the step's Jacobian in t is 2 z (times a
// reflection where a component is folded), so an error grows by |2 z| a
// step.  The roundings of different steps are independent, so their
// amplified errors add in quadrature (probabilistic rounding-error
// analysis: ~sqrt(n) eps after n steps where the worst case is n eps, which
// after 10^4 FP32 steps would already be 2^-8):
//   e2' = 4 |z|^2 e2 + |t'|^2,   err^2 = ke e2 2^(2e),   ke = 16 eps^2 K^2
// with K = 4 standard deviations.  A pixel is sent to the next pass
// (lost = 64) when err can change a decision (an escape test, a side of
// the fold) or, in FP32, when at a 4th iteration the relative error of t
// is above 2^-8 or the absolute error of z above 2^-12 (fold_checkpoint).
template <class T>
__device__ __forceinline__ T fold_ke(const PerturbLaunch&)
{
    return (T)(Mant<T>::kEps2x16 * 16.0);
}

template <class T>
__device__ __forceinline__ bool fold_err_hopeless(const PixState<T>& st)
{
    const T dd = Mant<T>::fma_(st.tr, st.tr, st.ti * st.ti);
    return !(st.ke * st.e2 <= (T)1.52587890625e-05 * dd) || !(st.kb * st.e2 <= (T)0.015625);
}

// The every-4th-iteration check.  A trajectory whose estimate passed the
// limits goes to the next pass, except in the FP64 pass of a folded
// formula: there it is marked `lost_track` and its later decisions are no
// longer sent to the multi-limb pass, since an error that large means the
// pixel's orbit is chaotic beyond what any fixed precision resolves (MPFR
// at the reference's precision and at twice it disagree there); such a
// pixel keeps its FP64 count, as the reference keeps its own.  (The
// Mandelbrot map is conformal: there a large estimate comes from rebases,
// and the multi-limb pass settles the pixel.)  Returns true when the pixel
// stops here, flagged.
template <class T, int FR>
__device__ __forceinline__ bool fold_checkpoint(const PerturbLaunch& p, const PixState<T>& st,
                                                float& lost, bool& lost_track)
{
    if (fold_err_hopeless(st)) {
        if (sizeof(T) == 4 || FR == MDZ_MANDELBROT)
            lost = fmaxf(lost, 64.f);
        else
            lost_track = true;
    }
    return lost > p.lost_limit && p.flag_out != nullptr;
}

// After a rebase (t, e replaced by Z_m + dz in FP64): the error carries
// over, plus the rounding of Z_m to FP64.
template <class T>
__device__ __forceinline__ void fold_rebase_err(const PerturbLaunch& p, int m, PixState<T>& st,
                                                int e0)
{
    const double2 zd = p.zd[m];
    const int ze = p.ze[m];
    const double z2 = zd.x * zd.x + zd.y * zd.y;
    const double add = ldexp(z2 * 4.930380657631324e-32 / (double)st.ke, 2 * (ze - st.e));
    st.e2 = (T)(ldexp((double)st.e2, 2 * (e0 - st.e)) + add);   // 2^-104 |Z|^2 above
}

// |z|^2 > 4 for a folded formula, exactly as escape_exact; `unsure` when
// |z|^2 - 4 is within the error estimate of z.
template <class T>
__device__ bool escape_fold(const PerturbLaunch& p, int m, const PixState<T>& st, bool& unsure)
{
    const double2 zd = p.zd[m];
    const int ze = p.ze[m];
    const double dd = p.dd[m];
    const int de = p.de[m];
    const double t2 = 2.0 * (zd.x * (double)st.tr + zd.y * (double)st.ti);
    const int e2 = ze + st.e;
    const double t3 = (double)st.tr * st.tr + (double)st.ti * st.ti;
    const int e3 = 2 * st.e;
    const int E = max(max(dexp_of(dd) + de, dexp_of(t2) + e2), dexp_of(t3) + e3);
    const double v = ldexp(dd, de - E) + ldexp(t2, e2 - E) + ldexp(t3, e3 - E);
    const double margin = ldexp(v, E);
    const double err = ldexp(sqrt((double)st.ke * (double)st.e2), st.e);
    unsure = !(fabs(margin) > err * (4.5 + err));
    return v > 0.0;
}

// One exact step of a folded formula in FP64 with exponents (dz below the
// FP32 range, |Z_m| tiny, or z near the fold): with c = F_m (the fold
// quantity of Z_m) and d its change, the folded part is
// |c + d| - |c| = sign(c) d while c + d keeps the sign of c, and
// -sign(c) (2c + d) when it crosses.  The side of the fold is decided from
// z = Z_m + dz in FP64; where even that can not decide it the pixel is
// marked (`lost`) for the multi-limb pass.
template <class T, int FR>
__device__ __forceinline__ void fold_step(const PerturbLaunch& p, int m, PixState<T>& st, T dcf_r,
                                          T dcf_i, double dcm_r, double dcm_i, int dce,
                                          float& lost)
{
    const double2 zd = p.zd[m];
    const int ze = p.ze[m];
    const double tr = (double)st.tr, ti = (double)st.ti;
    // unfolded pieces: a = 2 Z dz (exp ae), b = dz^2 (exp be)
    const double ar = 2.0 * (zd.x * tr - zd.y * ti), ai = 2.0 * (zd.x * ti + zd.y * tr);
    const int ae = ze + st.e;
    const double br = tr * tr - ti * ti, bi = 2.0 * tr * ti;
    const int be = 2 * st.e;
    // the fold quantity c = fm 2^fe and its exact sign
    const double fmv = p.fm[m];
    const int fev = p.fe[m];
    const double sc = (double)fold_sign(p, m);
    // side of the fold after adding dz.  Burning ship: the signs of
    // x = X + dx and y = Y + dy, each summed at its own exponent (a sign is
    // sure when the sum is not within FP64 rounding of its larger term).
    // Celtic: the sign of x^2 - y^2 = c + d, c exact from the digits, d from
    // the delta terms (sure when c + d is not within rounding of |c| + |d|).
    // Both tests also want the margin above the error estimate of z
    // (err = ea 2^e).
    const double eps = 1.4210854715202004e-14;  // 2^-46
    const double ea = sqrt((double)st.ke * (double)st.e2);
    double side;  // sign of the fold quantity of z
    bool sure;
    if (FR == MDZ_BURNING_SHIP) {
        const int Ex = max(dexp_of(zd.x) + ze, dexp_of(tr) + st.e);
        const int Ey = max(dexp_of(zd.y) + ze, dexp_of(ti) + st.e);
        const double xr = ldexp(zd.x, ze - Ex) + ldexp(tr, st.e - Ex);
        const double xi = ldexp(zd.y, ze - Ey) + ldexp(ti, st.e - Ey);
        side = ((xr < 0.0) != (xi < 0.0)) ? -1.0 : 1.0;
        sure = fabs(xr) > fmax(eps, ldexp(ea, st.e - Ex))
               && fabs(xi) > fmax(eps, ldexp(ea, st.e - Ey));
    } else {
        const int Es = max(max(dexp_of(fmax(fabs(ar), fabs(ai))) + ae,
                               dexp_of(fmax(fabs(br), fabs(bi))) + be),
                           dexp_of(fmv) + fev);
        const double cs = ldexp(fmv, fev - Es);
        const double a1 = ldexp(ar, ae - Es), b1 = ldexp(br, be - Es);
        const double v = cs + (a1 + b1);
        side = v < 0.0 ? -1.0 : 1.0;
        // | |x|^2 - |y|^2 | moves by at most 2 sqrt2 |z| err + 2 err^2
        sure = fabs(v) > eps * (fabs(cs) + fabs(a1) + fabs(b1))
               && fabs(v) > ldexp(ea, st.e - Es) * (6.0 + ldexp(ea, st.e));
    }
    if (!sure)
        lost += 64.f;  // undecidable here: the next pass redoes it
    const bool cross = side != sc;
    // pieces at a common exponent E: the folded component is
    //   sc * d            (no crossing)   or   -sc * (2c + d)   (crossing)
    // with d = (a + b) (celtic: real parts; ship: imaginary parts / 2 ... x2)
    double fr_, fi_;   // folded component terms
    int E = max(max(dexp_of(fmax(fabs(ar), fabs(ai))) + ae,
                    dexp_of(fmax(fabs(br), fabs(bi))) + be),
                dexp_of(fmax(fabs(dcm_r), fabs(dcm_i))) + dce);
    if (cross && fmv != 0.0)
        E = max(E, dexp_of(fmv) + fev + 2);
    double rr, ri;
    if (FR == MDZ_BURNING_SHIP) {
        // Re: unfolded; Im: 2 (|c + d| - |c|) with d = Z_re dz_im + dz_re Z_im + dz_re dz_im
        rr = ldexp(ar, ae - E) + ldexp(br, be - E) + ldexp(dcm_r, dce - E);
        const double dd2 = ldexp(ai, ae - E) + ldexp(bi, be - E);   // = 2 d
        fi_ = cross ? -sc * (ldexp(fmv, fev + 2 - E) + dd2) : sc * dd2;
        ri = fi_ + ldexp(dcm_i, dce - E);
        (void)fr_;
    } else {
        // Re: |c + d| - |c| with d = 2 Re(Z dz) + Re(dz^2); Im: unfolded
        const double d = ldexp(ar, ae - E) + ldexp(br, be - E);
        fr_ = cross ? -sc * (ldexp(fmv, fev + 1 - E) + d) : sc * d;
        rr = fr_ + ldexp(dcm_r, dce - E);
        ri = ldexp(ai, ae - E) + ldexp(bi, be - E) + ldexp(dcm_i, dce - E);
        (void)fi_;
    }
    set_from_double(st, rr, ri, E);
    refresh_scale(st, dcf_r, dcf_i, dce);
}

// Per-block copy of the orbit progress: pixel threads read shared memory;
// one elected thread at a time refreshes it from global memory, so the
// hundreds of thousands of waiting threads do not hammer one L2 line (which
// would also slow the producer's fences).
struct BlockOrbitView {
    int fin;    // finished entries (>= 2 once valid)
    int len;    // final length, 0 while the producer runs
    int busy;   // a thread is refreshing
};

__device__ __forceinline__ bool wait_orbit(const PerturbLaunch& p, BlockOrbitView* v, int need,
                                           int& avail, int& K)
{
    int spins = 0;
    for (;;) {
        const int f = *(volatile int*)&v->fin;
        const int len = *(volatile int*)&v->len;
        if (len && f >= len) {
            avail = f;
            K = len;
            __threadfence();
            return true;
        }
        if (f > need) {
            avail = f;
            __threadfence();  // acquire: the entries below f are visible
            return true;
        }
        if (atomicCAS(&v->busy, 0, 1) == 0) {
            const int gf = *(volatile const int*)p.fin_len;
            const int gd = *(volatile const int*)p.orbit_done;
            const int gl = gd ? *(volatile const int*)p.orbit_len : 0;
            if (gf > *(volatile int*)&v->fin)
                *(volatile int*)&v->fin = gf;
            if (gl)
                *(volatile int*)&v->len = gl;
            __threadfence_block();
            atomicExch(&v->busy, 0);
        }
        if (*(volatile const int*)p.orbit_error || ++spins > p.spin_limit) {
            atomicExch(p.orbit_error, 1);
            return false;
        }
        __nanosleep(256);
    }
}

// Resumable state of one pixel: the deltas, the reference index m, the next
// iteration wz, the bits lost to rebases so far.  (s, s2scr, dc 2^-e and the
// flags follow from t, e and dc, so they are recomputed on resume and a
// resumed run is bit-identical to an uninterrupted one.)
template <class T>
struct PixRun {
    PixState<T> st;
    int m;
    uint32_t wz;
    float lost;
    unsigned rebases;
    float mag;
};

template <class T>
__device__ __forceinline__ void pixel_start(PixRun<T>& r, double dcm_r, double dcm_i, int dce,
                                            T ke)
{
    set_from_double(r.st, dcm_r, dcm_i, dce);
    r.st.ke = ke;
    r.st.e2 = Mant<T>::fma_(r.st.tr, r.st.tr, r.st.ti * r.st.ti);  // the rounding of dc 2^-e
    refresh_scale(r.st, (T)dcm_r, (T)dcm_i, dce);
    r.m = 1;
    r.wz = 1;
    r.lost = 0.f;
    r.rebases = 0;
    r.mag = 0.f;
}

// The hot step t' = 2 Z_m t + s t^2 + dc 2^-e.  Variant 2 (the default)
// keeps the two products apart: s t^2 is added to dc first, then each
// 2 Z_m t term enters through an FMA with its exact product (11 FP32 ops).
// Variants 0 / 1 factor it as t (2 Z_m + s t) (6 / 8 ops) and round
// w = 2 Z_m + s t before the product; on the gallery views that extra
// rounding moved 3 of 1728 pixels off the 2x-precision MPFR counts (variant
// 2: 1), so the factored forms stay opt-in (-DMDZ_STEP_VARIANT=0/1).
#ifndef MDZ_STEP_VARIANT
#define MDZ_STEP_VARIANT 2
#endif
template <class T>
__device__ __forceinline__ void fast_step(PixState<T>& st, T Zx, T Zy, T zr, T zi)
{
    const T tr = st.tr, ti = st.ti;
#if MDZ_STEP_VARIANT == 0
    const T wr = zr + Zx, wi = zi + Zy;
    st.tr = Mant<T>::fma_(tr, wr, Mant<T>::fma_(-ti, wi, st.dcr));
    st.ti = Mant<T>::fma_(tr, wi, Mant<T>::fma_(ti, wr, st.dci));
#elif MDZ_STEP_VARIANT == 1
    const T wr = Mant<T>::fma_(Zx, (T)2, st.s * tr), wi = Mant<T>::fma_(Zy, (T)2, st.s * ti);
    st.tr = Mant<T>::fma_(tr, wr, Mant<T>::fma_(-ti, wi, st.dcr));
    st.ti = Mant<T>::fma_(tr, wi, Mant<T>::fma_(ti, wr, st.dci));
#else
    const T u = tr + tr, v = ti + ti;
    const T a = Mant<T>::fma_(tr, tr, -ti * ti);
    const T b = tr * v;
    st.tr = Mant<T>::fma_(Zx, u, Mant<T>::fma_(-Zy, v, Mant<T>::fma_(st.s, a, st.dcr)));
    st.ti = Mant<T>::fma_(Zx, v, Mant<T>::fma_(Zy, u, Mant<T>::fma_(st.s, b, st.dci)));
#endif
}

// The FP32 / FP64 step of a folded formula away from its fold: the folded
// component's change is sign(F_m) times the unfolded one (burning ship:
// Im = 2 |Re Im| + Ci; celtic: Re = |Re^2 - Im^2| + Cr), the other
// component is Mandelbrot's.
template <class T, int FR>
__device__ __forceinline__ void fold_fast_step(PixState<T>& st, T Zx, T Zy, T fs)
{
    const T tr = st.tr, ti = st.ti;
    const T u = tr + tr, v = ti + ti;
    const T a = Mant<T>::fma_(tr, tr, -ti * ti);
    const T b = tr * v;
    if (FR == MDZ_BURNING_SHIP) {
        st.tr = Mant<T>::fma_(Zx, u, Mant<T>::fma_(-Zy, v, Mant<T>::fma_(st.s, a, st.dcr)));
        const T w = Mant<T>::fma_(Zx, v, Mant<T>::fma_(Zy, u, st.s * b));
        st.ti = Mant<T>::fma_(fs, w, st.dci);
    } else {
        const T w = Mant<T>::fma_(Zx, u, Mant<T>::fma_(-Zy, v, st.s * a));
        st.tr = Mant<T>::fma_(fs, w, st.dcr);
        st.ti = Mant<T>::fma_(Zx, v, Mant<T>::fma_(Zy, u, Mant<T>::fma_(st.s, b, st.dci)));
    }
}

// Float pair ("double-float"): a value hi + lo with |lo| <= ulp(hi) / 2,
// about 48 significant bits, from FP32 operations only (Dekker's and Knuth's
// error-free transformations: the product's rounding error from one FMA, the
// sum's from the two-sum sequence).  On this GPU an FP64 operation costs as
// much issue time as ~64 FP32 ones, so a pair step (about 70 FP32
// operations) is several times cheaper than the FP64 step it replaces.
struct FPair {
    float hi, lo;
};

__device__ __forceinline__ FPair fp_from(double d)
{
    const float h = __double2float_rn(d);
    return FPair{h, __double2float_rn(d - (double)h)};
}

// a + b with |a| >= |b| (or a == 0): exact as a pair
__device__ __forceinline__ FPair fp_quick(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return FPair{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ FPair fp_add(FPair a, FPair b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return fp_quick(s, e);
}

__device__ __forceinline__ FPair fp_mul(FPair a, FPair b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fp_quick(p, e);
}

__device__ __forceinline__ FPair fp_neg(FPair a)
{
    return FPair{-a.hi, -a.lo};
}

__device__ __forceinline__ FPair fp_abs(FPair a)
{
    return a.hi < 0.f ? fp_neg(a) : a;
}

__device__ __forceinline__ FPair fp_twice(FPair a)
{
    return FPair{a.hi + a.hi, a.lo + a.lo};
}

// The rest of a folded-formula pixel whose FP64 error estimate is lost
// (its orbit is chaotic beyond the pass's precision): the deltas no longer
// carry the pixel's offset from the reference (the error is far above dc),
// so its own orbit z' = f(z) + c is iterated directly, which gives the same
// kind of trajectory without the rebases and orbit reads that perturbation
// needs once z is far from the reference.  The iteration runs in float
// pairs (~48 bits; FP64 would resolve such an orbit no better, its error
// having already passed the estimate's limit, and costs ~6x the issue
// time).  z = z_wz; runs iterations wz + 1 .. depth.  Returns the count
// (0: did not escape).
template <int FR>
__device__ uint32_t fold_direct(double xr0, double xi0, double cr0, double ci0, uint32_t wz,
                                uint32_t depth, float& mag)
{
    FPair xr = fp_from(xr0), xi = fp_from(xi0);
    const FPair cr = fp_from(cr0), ci = fp_from(ci0);
    for (uint32_t w = wz + 1; w <= depth; ++w) {
        const FPair x2 = fp_mul(xr, xr), y2 = fp_mul(xi, xi);
        const FPair a = fp_add(x2, fp_neg(y2));
        const FPair b = fp_mul(xr, xi);
        if (FR == MDZ_BURNING_SHIP) {
            xr = fp_add(a, cr);
            xi = fp_add(fp_twice(fp_abs(b)), ci);
        } else if (FR == MDZ_VARIANT && !(w & 1u)) {
            xr = fp_add(a, cr);   // the hybrid's even iterations are Mandelbrot's
            xi = fp_add(fp_twice(b), ci);
        } else {
            xr = fp_add(fp_abs(a), cr);
            xi = fp_add(fp_twice(b), ci);
        }
        const FPair m2 = fp_add(fp_mul(xr, xr), fp_mul(xi, xi));
        if (m2.hi > 4.f || (m2.hi == 4.f && m2.lo > 0.f)) {
            mag = m2.hi;
            return w;
        }
    }
    mag = __fmaf_rn(xr.hi, xr.hi, xi.hi * xi.hi);
    return 0;
}

// How a pixel learns which reference-orbit entries it may read:
//   kOrbitComplete  the orbit is finished: K = *orbit_len entries;
//   kOrbitWait      fused launch: wait (bounded) for the finisher;
//   kOrbitSnapshot  entries below snap.avail are finished (K = snap.K, or
//                   INT_MAX while the producer runs); a pixel that needs a
//                   later entry stops and is resumed in a later step.
enum { kOrbitComplete = 0, kOrbitWait = 1, kOrbitSnapshot = 2 };

struct OrbitSnap {
    int avail;
    int K;
};

// Orbit progress as a step sees it (read once per pixel visit).
__device__ __forceinline__ OrbitSnap orbit_snapshot(const PerturbLaunch& p)
{
    OrbitSnap s;
    const int done = *(volatile const int*)p.orbit_done;
    s.K = done ? *(volatile const int*)p.orbit_len : 0x7fffffff;
    s.avail = *(volatile const int*)p.fin_len;
    return s;
}

// Iterations r.wz .. wz_last (inclusive, <= depth).  Returns 1 when the
// pixel is finished (*count = escape iteration, or 0 at depth), 0 when it
// stopped after wz_last or (snapshot mode) at the last finished orbit entry
// (state in r), -1 when an orbit wait gave up.
//
// One iteration (dz = t 2^e, s = 2^e, z = Z_m + dz):
//   w  = z + Z_m                        (= 2 Z_m + s t; z carried from the
//                                         previous iteration's escape test)
//   t' = t w + dc 2^-e                  (4 FMA: the complex product)
//   m += 1;  z' = Z_m + s t'  (2 FMA),  |z'|^2 (2)
//   attention when |z'|^2 > 4 - 2^-14 (escape band) or
//   |z'|^2 <= (1 + 2^-16) |dz'|^2 (the rebase screen; the exact FP64 test
//   decides) or |z'| tiny.
// Iterations 4k+1 .. 4k+4 whose orbit entries are all finished run as one
// unrolled block without the orbit, budget and rescale checks; the block
// leaves at the first iteration that needs attention and that iteration
// continues on the general path, so the operations are the same whether a
// pixel runs in blocks or not, and a pixel resumed at any iteration gets
// bit-identical results.
template <class T, int MODE, int FR = MDZ_MANDELBROT, bool JU = false>
__device__ int perturb_run(const PerturbLaunch& p, PixRun<T>& r, double dcm_r, double dcm_i,
                           int dce, uint32_t wz_last, uint32_t& count, BlockOrbitView* view,
                           OrbitSnap snap = OrbitSnap{0, 0})
{
    const T dcf_r = (T)dcm_r, dcf_i = (T)dcm_i;
    PixState<T>& st = r.st;
    int m = r.m;
    // entries 0..avail-1 readable; K = orbit length (unknown while streaming)
    int K = MODE == kOrbitComplete ? *p.orbit_len : (MODE == kOrbitSnapshot ? snap.K : 0x7fffffff);
    int avail = MODE == kOrbitSnapshot ? snap.avail : K;
    // Julia and the hybrid carry two orbits: K ends the segment the pixel
    // is on (the first, or the second from q0)
    constexpr bool kVar = FR == MDZ_VARIANT;
    constexpr bool kTwo = JU || kVar;
    const int q0 = kTwo ? p.q0 : 0;
    if (kTwo) {
        K = m < q0 ? *p.orbit_len : q0 + *p.q_len;
        avail = K;
    }
    // where a rebase goes when iteration `next` steps from it: Julia: the
    // critical orbit; the hybrid: the orbit that folds at the parity of
    // `next` (the first folds at odd steps); else Z_0
    auto rebase_to = [&](uint32_t next) -> int {
        if (JU)
            return q0;
        if (kVar)
            return (next & 1u) ? q0 : 0;
        return 0;
    };
    if (MODE == kOrbitWait && !wait_orbit(p, view, m, avail, K))
        return -1;
    if (MODE == kOrbitSnapshot && m >= avail)
        return 0;  // Z_m not finished yet
    T Zx, Zy;
    load_z<T>(p, m, Zx, Zy);
    T fs = (T)1;   // fold sign of Z_m (burning ship / celtic)
    if (FR != MDZ_MANDELBROT)
        fs = (T)fold_sign(p, m);
    T zr = Mant<T>::fma_(st.s, st.tr, Zx);
    T zi = Mant<T>::fma_(st.s, st.ti, Zy);
    const T band_lo = (T)4 - (T)6.1035156e-5;  // 4 - 2^-14
    const T band_hi = (T)4 + (T)6.1035156e-5;
    T magT = (T)r.mag;
    // error estimate (see fold_ke), carried by the folded formulas and by
    // every FP64 pass: it grows by 4 |z|^2 (|z|^2 of the z about to be
    // stepped) and also covers what rebases cancel.  The FP32 Mandelbrot
    // pass counts the bits its rebases cancel instead.
    constexpr bool kTrack = FR != MDZ_MANDELBROT || sizeof(T) == 8;
    const T grow = (T)4;
    bool lost_track = false;   // FP64: the estimate passed its limits
    float lost_sink = 0.f;
    float& rebase_lost = kTrack ? lost_sink : r.lost;
    if (kTrack)
        magT = Mant<T>::fma_(zr, zr, zi * zi);
    const uint32_t last = wz_last < p.depth ? wz_last : p.depth;
    uint32_t wz = r.wz;
    bool blocked = false;
    while (wz <= last) {
        bool attention = false;
        // blocks: FP32 (the FP64 pass is the rare escalation path), no
        // slow step among the four (dz below the FP32 range needs one only
        // where Z_m is tiny)
        if (FR != MDZ_MANDELBROT && !kVar && sizeof(T) == 4 && (wz & 3u) == 1u
            && wz + 3u <= last && m + 4 < avail && st.s == (T)0 && !st.force_slow
            && four_not_axis(p, m)) {
            // folded formulas at deep zoom: z = Z_m in FP32 and no fold
            // within reach of dz among these entries, so the fold keeps
            // Z_m's side; same values as the general step with s = 0
            // with 2 Z from the orbit copy: 2Z t is Z (2t) exactly
            T Z2x = Zx + Zx, Z2y = Zy + Zy;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const T tr = st.tr, ti = st.ti;
                const T g = grow * magT;
                if (FR == MDZ_BURNING_SHIP) {
                    st.tr = Mant<T>::fma_(Z2x, tr, Mant<T>::fma_(-Z2y, ti, st.dcr));
                    st.ti = Mant<T>::fma_(fs, Mant<T>::fma_(Z2x, ti, Z2y * tr), st.dci);
                } else {
                    st.tr = Mant<T>::fma_(fs, Mant<T>::fma_(Z2x, tr, -Z2y * ti), st.dcr);
                    st.ti = Mant<T>::fma_(Z2x, ti, Mant<T>::fma_(Z2y, tr, st.dci));
                }
                st.e2 = Mant<T>::fma_(g, st.e2, Mant<T>::fma_(st.tr, st.tr, st.ti * st.ti));
                ++m;
                const float4 q = p.zq[m];
                Z2x = (T)q.x;
                Z2y = (T)q.y;
                magT = (T)q.z;
                fs = (T)q.w;
                if (magT > band_lo || magT < (T)Mant<T>::kGlitchZ2) {
                    attention = true;
                    break;
                }
                ++wz;
            }
            Zx = (T)0.5 * Z2x;
            Zy = (T)0.5 * Z2y;
            // the current z for the fold test of the general step (= Z_m)
            zr = Mant<T>::fma_(st.s, st.tr, Zx);
            zi = Mant<T>::fma_(st.s, st.ti, Zy);
            if (!attention) {
                const T amax = fmax(fabs(st.tr), fabs(st.ti));
                if ((amax > (T)4.2949673e9 || amax < (T)2.3283064e-10) && amax != (T)0) {
                    const int k = Mant<T>::exponent_of(amax);
                    const T sc = Mant<T>::scale((T)1, -k);
                    st.tr *= sc;
                    st.ti *= sc;
                    st.e += k;
                    st.e2 = Mant<T>::scale(st.e2, -2 * k);
                    refresh_scale(st, dcf_r, dcf_i, dce);
                    zr = Mant<T>::fma_(st.s, st.tr, Zx);
                    zi = Mant<T>::fma_(st.s, st.ti, Zy);
                }
                if (fold_checkpoint<T, FR>(p, st, r.lost, lost_track)) {
                    r.mag = (float)magT;
                    count = 0;
                    return 1;  // the next pass redoes the pixel
                }
                continue;
            }
        } else if (FR == MDZ_MANDELBROT && sizeof(T) == 4 && (wz & 3u) == 1u && wz + 3u <= last
                   && m + 4 < avail && !st.force_slow
                   && (!st.slow_if_tiny || four_not_tiny(p, m))) {
            // iterations wz .. wz+3, orbit entries m+1 .. m+4 all finished
            if (st.s == (T)0 && p.att && five_clear(p.att, m)) {
                const int mstart = m;
                // deep zoom and none of Z_m .. Z_{m+4} needs attention
                // (escape band, rebase screen, tiny |Z|): whole blocks of
                // four run with no test inside, their four orbit loads issued
                // together; the values are those of the checked block below
                // (the checks it makes would all have passed)
                // iteration wz steps from entry m, so wz - m stays fixed: both
                // bounds (wz + 3 <= last, m + 4 < avail) become one on m
                const int span = (int)min(last - wz, 0x3fffffffu);
                const int mmax = min(span + m - 3, avail - 5);
                // the clear run of the attention mask: no bit is set in
                // [m, nxt); `hit` when bit nxt is set, else nxt ends the last
                // mask word read.  A block may start at m while m + 4 < nxt
                // (five_clear(m)), so the loop runs while m <= lim; the run
                // is extended a word at a time, reading only words that hold
                // finished entries (nxt < avail; the finisher publishes
                // whole lines of the mask).
                const unsigned w0 = __ldg(p.att + (m >> 5)) & (0xffffffffu << (m & 31));
                bool hit = w0 != 0u;
                int nxt = hit ? (m & ~31) + __ffs(w0) - 1 : (m & ~31) + 32;
                auto extend = [&]() {
                    while (!hit && nxt <= m + 4 && nxt < avail) {
                        const unsigned w = __ldg(p.att + (nxt >> 5));
                        hit = w != 0u;
                        nxt += hit ? __ffs(w) - 1 : 32;
                    }
                    return min(mmax, nxt - 5);
                };
                int lim = extend();
                T Z2x = Zx + Zx, Z2y = Zy + Zy;
                // blocks counted down to the run's end; entries read through
                // a pointer (immediate offsets); a block after which |t| left
                // [2^-32, 2^32] ends the loop and the rescale follows it (the
                // rescale is exact, a power of two: where it happens changes
                // no value, and the next pass through here carries on)
                const float4* zp = p.zq + m;
                bool out = false;
                for (;;) {
                    int nb = (lim - m) / 4 + 1;
                    do {
                        const float4 q1 = zp[1], q2 = zp[2], q3 = zp[3], q4 = zp[4];
                        const T zx[4] = {Z2x, (T)q1.x, (T)q2.x, (T)q3.x};
                        const T zy[4] = {Z2y, (T)q1.y, (T)q2.y, (T)q3.y};
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            // t' = 2 Z t + dc 2^-e (as the checked block: 2Z t = Z (2t))
                            const T tr = st.tr, ti = st.ti;
                            st.tr = Mant<T>::fma_(zx[u], tr, Mant<T>::fma_(-zy[u], ti, st.dcr));
                            st.ti = Mant<T>::fma_(zx[u], ti, Mant<T>::fma_(zy[u], tr, st.dci));
                        }
                        Z2x = (T)q4.x;
                        Z2y = (T)q4.y;
                        magT = (T)q4.z;
                        zp += 4;
                        // wz - 1 = 4k + 4: the rescale check of the general path
                        const T amax = fmax(fabs(st.tr), fabs(st.ti));
                        out = (amax > (T)4.2949673e9 || amax < (T)2.3283064e-10) && amax != (T)0;
                    } while (--nb > 0 && !out);
                    m = (int)(zp - p.zq);
                    if (out || (lim = extend()) < m)
                        break;
                }
                if (out) {
                    const T amax = fmax(fabs(st.tr), fabs(st.ti));
                    const int k = Mant<T>::exponent_of(amax);
                    const T sc = Mant<T>::scale((T)1, -k);
                    st.tr *= sc;
                    st.ti *= sc;
                    st.e += k;
                    refresh_scale(st, dcf_r, dcf_i, dce);
                }
                wz += (uint32_t)(m - mstart);
                Zx = (T)0.5 * Z2x;
                Zy = (T)0.5 * Z2y;
                // as a resumed pixel computes it
                zr = Mant<T>::fma_(st.s, st.tr, Zx);
                zi = Mant<T>::fma_(st.s, st.ti, Zy);
                continue;
            }
            if (st.s == (T)0) {
                // dz below the FP32 range (deep zoom): s t and s t^2 vanish
                // exactly, so the step is t' = 2 Z_m t + dc 2^-e, |z|^2 is
                // |Z_m|^2 (stored with the entry, formed as below) and the
                // rebase screen is |z| tiny -- the same values the general
                // code computes with s = 0
                T Z2x = Zx + Zx, Z2y = Zy + Zy;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const T tr = st.tr, ti = st.ti;
                    st.tr = Mant<T>::fma_(Z2x, tr, Mant<T>::fma_(-Z2y, ti, st.dcr));
                    st.ti = Mant<T>::fma_(Z2x, ti, Mant<T>::fma_(Z2y, tr, st.dci));
                    ++m;
                    const float4 q = p.zq[m];
                    Z2x = (T)q.x;
                    Z2y = (T)q.y;
                    magT = (T)q.z;
                    if (magT > band_lo || magT < (T)Mant<T>::kGlitchZ2) {
                        attention = true;
                        break;
                    }
                    ++wz;
                }
                Zx = (T)0.5 * Z2x;
                Zy = (T)0.5 * Z2y;
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    fast_step<T>(st, Zx, Zy, zr, zi);
                    ++m;
                    load_z<T>(p, m, Zx, Zy);
                    zr = Mant<T>::fma_(st.s, st.tr, Zx);
                    zi = Mant<T>::fma_(st.s, st.ti, Zy);
                    magT = Mant<T>::fma_(zr, zr, zi * zi);
                    const T dd = Mant<T>::fma_(st.tr, st.tr, st.ti * st.ti);
                    if (magT > band_lo || Mant<T>::fma_(st.s2scr, dd, -magT) >= (T)0
                        || magT < (T)Mant<T>::kGlitchZ2) {
                        attention = true;
                        break;
                    }
                    ++wz;
                }
            }
            if (!attention) {
                // wz - 1 = 4k + 4: the rescale check of the general path
                const T amax = fmax(fabs(st.tr), fabs(st.ti));
                if ((amax > (T)4.2949673e9 || amax < (T)2.3283064e-10) && amax != (T)0) {
                    const int k = Mant<T>::exponent_of(amax);
                    const T sc = Mant<T>::scale((T)1, -k);
                    st.tr *= sc;
                    st.ti *= sc;
                    st.e += k;
                    refresh_scale(st, dcf_r, dcf_i, dce);
                    // as a resumed pixel computes it
                    zr = Mant<T>::fma_(st.s, st.tr, Zx);
                    zi = Mant<T>::fma_(st.s, st.ti, Zy);
                }
                continue;
            }
            // iteration wz is stepped; it continues below
        } else {
            if (m + 1 >= avail) {
                if (MODE == kOrbitWait && m + 1 < K && !wait_orbit(p, view, m + 1, avail, K))
                    return -1;
                if (MODE == kOrbitSnapshot && m + 1 < K) {
                    blocked = true;  // Z_{m+1} not finished: resume in a later step
                    break;
                }
                if (m >= K - 1) {
                    // end of the reference orbit: rebase onto Z_0 = 0
                    const int e0 = st.e;
                    rebase_fp64<T>(p, m, st, dcf_r, dcf_i, dce, rebase_lost, false);
                    if (kTrack)
                        fold_rebase_err<T>(p, m, st, e0);
                    m = rebase_to(wz);
                    if (kTwo)
                        K = avail = m ? q0 + *p.q_len : *p.orbit_len;
                    Zx = (T)0;
                    Zy = (T)0;
                    fs = (T)1;
                    zr = Mant<T>::fma_(st.s, st.tr, Zx);
                    zi = Mant<T>::fma_(st.s, st.ti, Zy);
                    if (kTrack)
                        magT = Mant<T>::fma_(zr, zr, zi * zi);
                    ++r.rebases;
                }
            }
            const bool careful = st.careful && (st.force_slow || z_tiny<T>(p, m, Zx, Zy));
            // stepping from a reference entry at zero other than the orbit's
            // start (the view is centred on a minibrot's nucleus, Z_p = 0):
            // the FP64 pass redoes the pixel (see kFp32AtZeroLost), so this
            // pass stops here
            if (!kTrack && m != 0 && !(kTwo && m == q0) && z_tiny<T>(p, m, Zx, Zy)) {
                r.lost = fmaxf(r.lost, kFp32AtZeroLost);
                if (p.flag_out) {
                    r.mag = 0.f;
                    count = 0;
                    return 1;
                }
            }
            const T g = kTrack ? grow * magT : (T)0;
            // the hybrid folds on odd iterations only
            if (FR != MDZ_MANDELBROT && (!kVar || (wz & 1u))) {
                // with dz below the T range (s = 0) a fold is out of reach
                // unless the entry is marked: the same choice as the blocks
                // (a lost estimate leaves only the rounding margin: the side
                // is still decided exactly, its error no longer matters)
                const bool fast =
                    !careful && !axis_bit(p, m)
                    && (st.s == (T)0
                        || fold_certain<T, FR>(
                            zr, zi, Zx, Zy, fs,
                            lost_track ? (T)0 : st.sm * fmax(fabs(st.tr), fabs(st.ti))));
                if (fast) {
                    fold_fast_step<T, FR>(st, Zx, Zy, fs);
                } else {
                    const int e0 = st.e;
                    float unsure = 0.f;
                    fold_step<T, FR>(p, m, st, dcf_r, dcf_i, dcm_r, dcm_i, dce, unsure);
                    if (!lost_track)
                        r.lost += unsure;
                    if (st.e != e0)
                        st.e2 = Mant<T>::scale(st.e2, 2 * (e0 - st.e));
                }
            } else if (careful) {
                const int e0 = st.e;
                slow_step<T>(p, m, st, dcf_r, dcf_i, dcm_r, dcm_i, dce);
                if (kTrack && st.e != e0)
                    st.e2 = Mant<T>::scale(st.e2, 2 * (e0 - st.e));
            } else {
                fast_step<T>(st, Zx, Zy, zr, zi);
            }
            ++m;
            load_z<T>(p, m, Zx, Zy);
            if (FR != MDZ_MANDELBROT)
                fs = (T)fold_sign(p, m);
            zr = Mant<T>::fma_(st.s, st.tr, Zx);
            zi = Mant<T>::fma_(st.s, st.ti, Zy);
            magT = Mant<T>::fma_(zr, zr, zi * zi);
            if (kTrack)
                st.e2 = Mant<T>::fma_(g, st.e2, Mant<T>::fma_(st.tr, st.tr, st.ti * st.ti));
        }
        if (kTrack) {
            // the band widens to 2^9 err where the error estimate of z is
            // larger (not once the estimate is lost: its decisions stand)
            const T dv = magT - (T)4;
            if (dv > -(T)6.1035156e-5 || (!lost_track && dv * dv <= st.kb * st.e2)) {
                bool unsure;
                const bool esc = escape_fold<T>(p, m, st, unsure);
                if (unsure && !lost_track)
                    r.lost = fmaxf(r.lost, 64.f);
                if (esc) {
                    r.mag = (float)magT;
                    count = wz;
                    return 1;
                }
            }
        } else if (magT > band_lo) {
            // within 2^-14 of the bailout the rounded Z_m can not decide it
            if (magT > band_hi || escape_exact<T>(p, m, st)) {
                r.mag = (float)magT;
                count = wz;
                return 1;
            }
        }
        // rebase when |Z_m + dz| < |dz|, decided exactly in FP64; the screen
        // in T passes |z|^2 <= (1 + 2^-16) |dz|^2 (or |z| tiny) to it.  Where
        // the screen stops a pixel, |z| > |dz| and so |Z_m| < 2 |z|: z in T
        // (Z_m rounded, one FMA) is off by at most 2^-24 (|Z_m| + |z|) a
        // component, |z|^2 and |dz|^2 by under 2^-20 relative, and the FP64
        // test would not rebase either.  (Once a pixel has left the
        // reference, |z| and |dz| are alike in size and a screen as loose
        // as |z| <= 2 |dz| sent most of its steps through FP64.)
        const T dd = Mant<T>::fma_(st.tr, st.tr, st.ti * st.ti);
        if (Mant<T>::fma_(st.s2scr, dd, -magT) >= (T)0 || magT < (T)Mant<T>::kGlitchZ2) {
            const int e0 = st.e;
            if (rebase_fp64<T>(p, m, st, dcf_r, dcf_i, dce, rebase_lost, true)) {
                if (kTrack)
                    fold_rebase_err<T>(p, m, st, e0);
                m = rebase_to(wz + 1);
                if (kTwo)
                    K = avail = m ? q0 + *p.q_len : *p.orbit_len;
                Zx = (T)0;
                Zy = (T)0;
                fs = (T)1;
                zr = Mant<T>::fma_(st.s, st.tr, Zx);
                zi = Mant<T>::fma_(st.s, st.ti, Zy);
                if (kTrack)
                    magT = Mant<T>::fma_(zr, zr, zi * zi);
                ++r.rebases;
                ++wz;
                continue;
            }
        }
        // keep |t| in [2^-32, 2^32]; it changes by at most ~2^3 a step, so
        // checking every 4th step is enough
        if ((wz & 3u) == 0u) {
            const T amax = fmax(fabs(st.tr), fabs(st.ti));
            if ((amax > (T)4.2949673e9 || amax < (T)2.3283064e-10) && amax != (T)0) {
                const int k = Mant<T>::exponent_of(amax);
                const T sc = Mant<T>::scale((T)1, -k);
                st.tr *= sc;
                st.ti *= sc;
                st.e += k;
                if (kTrack)
                    st.e2 = Mant<T>::scale(st.e2, -2 * k);
                refresh_scale(st, dcf_r, dcf_i, dce);
                zr = Mant<T>::fma_(st.s, st.tr, Zx);
                zi = Mant<T>::fma_(st.s, st.ti, Zy);
            }
            if (kTrack && fold_checkpoint<T, FR>(p, st, r.lost, lost_track)) {
                r.mag = (float)magT;
                count = 0;
                return 1;  // the next pass redoes the pixel
            }
            if (FR != MDZ_MANDELBROT && sizeof(T) == 8 && MODE == kOrbitComplete && lost_track
                && last == p.depth) {
                // c = Z_1 + dc
                const double cr = ldexp(p.zd[1].x, p.ze[1]) + ldexp(dcm_r, dce);
                const double ci = ldexp(p.zd[1].y, p.ze[1]) + ldexp(dcm_i, dce);
                float mg = 0.f;
                count = fold_direct<FR>((double)zr, (double)zi, cr, ci, wz, p.depth, mg);
                r.mag = mg;
                r.m = m;
                r.wz = p.depth + 1;
                return 1;
            }
        }
        ++wz;
    }
    r.mag = (float)magT;
    r.m = m;
    r.wz = wz;
    if (!blocked && wz > p.depth) {
        count = 0;
        return 1;
    }
    return 0;
}

// One pixel.  Returns the count; mag_out gets |z|^2 at escape.  `lost`
// accumulates the bits cancelled by rebases (log2 |dz| / |z| at each one):
// a pixel whose deltas lost more than the mantissa can spare is re-run by
// the next, more precise, pass.
// In the fused launch (STREAM) the orbit is still being produced: entries
// below `avail` are finished; a pixel that needs entry m + 1 waits (bounded)
// for the finisher, and learns the final length K once the producer is done.
// A wait that gives up raises the error flag and leaves the count 0.
template <class T, bool STREAM, int FR, bool JU = false>
__device__ uint32_t perturb_pixel(const PerturbLaunch& p, double dcm_r, double dcm_i, int dce,
                                  float& mag_out, unsigned& rebases, float& lost,
                                  BlockOrbitView* view)
{
    PixRun<T> r;
    pixel_start(r, dcm_r, dcm_i, dce, fold_ke<T>(p));
    if (JU) {
        // Julia: the offset is the first delta, at V_0; no dc in the steps
        r.m = 0;
        refresh_scale(r.st, (T)0, (T)0, dce);
    }
    uint32_t count = 0;
    const int done = perturb_run<T, STREAM ? kOrbitWait : kOrbitComplete, FR, JU>(
        p, r, JU ? 0.0 : dcm_r, JU ? 0.0 : dcm_i, dce, p.depth, count, view);
    mag_out = r.mag;
    rebases += r.rebases;
    lost += r.lost;
    return done == 1 ? count : 0;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Frame pass (FP32): 8x4 tiles per warp from the atomic counter.  Pass 2
// (FP64) walks the list of pixels the previous pass flagged, in warp-sized
// chunks.  Each pass appends the pixels it could not finish precisely to
// p.flag_out; pixel-iterations are counted only for pixels it finalises.
template <class T, bool WANT_MAG, bool LIST, bool STREAM, int FR, bool JU = false>
__device__ __forceinline__ void pixel_tiles(const PerturbLaunch& p)
{
    __shared__ BlockOrbitView view;
    if (STREAM) {
        if (threadIdx.x == 0) {
            view.fin = 0;
            view.len = 0;
            view.busy = 0;
        }
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int tiles_x = (p.W + kTileW - 1) / kTileW;
    const int tiles_y = (p.nrows + kTileH - 1) / kTileH;
    const unsigned total = LIST ? (unsigned)((*p.list_in_count + 31) / 32)
                                : (unsigned)tiles_x * (unsigned)tiles_y;
    const unsigned list_n = LIST ? *p.list_in_count : 0u;
    for (;;) {
        unsigned tile = 0;
        if (lane == 0) {
            const unsigned t = (p.stop && *p.stop) ? 0xffffffffu
                                                    : atomicAdd(&p.sync->tile_counter, 1u);
            tile = t >= p.tile_limit ? total : p.tile_base + t;
        }
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= total)
            break;
        int ix, lrow;
        bool valid;
        if (LIST) {
            const unsigned i = tile * 32u + lane;
            valid = i < list_n;
            const unsigned pix = valid ? p.list_in[i] : 0u;
            lrow = (int)(pix / (unsigned)p.W);
            ix = (int)(pix - (unsigned)lrow * (unsigned)p.W);
        } else {
            const int ty = (int)(tile / (unsigned)tiles_x);
            const int tx = (int)(tile - (unsigned)ty * (unsigned)tiles_x);
            ix = tx * kTileW + (lane & (kTileW - 1));
            lrow = ty * kTileH + (lane / kTileW);
            valid = ix < p.W && lrow < p.nrows;
        }
        unsigned long long its = 0;
        unsigned reb = 0;
        if (valid) {
            const int line = p.row0 + lrow;
            // dc = ((2 ix - W) hs, (H - 2 line) hs), hs = half pixel spacing
            const double dcm_r = (double)(2 * ix - p.W) * p.hs_m;
            const double dcm_i = (double)(p.H - 2 * line) * p.hs_m;
            float mag = 0.f, lost = 0.f;
            const uint32_t n =
                perturb_pixel<T, STREAM, FR, JU>(p, dcm_r, dcm_i, p.hs_e, mag, reb, lost, &view);
            const size_t o = (size_t)lrow * p.W + ix;
            p.out[o] = (int32_t)n;
            if (WANT_MAG)
                p.mag[o] = mag;
            if (lost > p.lost_limit && p.flag_out) {
                const unsigned slot = atomicAdd(p.flag_out_count, 1u);
                p.flag_out[slot] = (unsigned)o;
            } else {
                its = n ? n : p.depth;
            }
        }
        its = warp_sum_u64(its);
        unsigned long long rb = warp_sum_u64((unsigned long long)reb);
        __syncwarp();
        if (lane == 0) {
            atomicAdd(&p.sync->iter_sum, its);
            if (rb)
                atomicAdd(p.rebases, rb);
        }
    }
}

template <class T, bool WANT_MAG, bool LIST, int FR, bool JU>
__global__ void __launch_bounds__(256) perturb_kernel(PerturbLaunch p)
{
    pixel_tiles<T, WANT_MAG, LIST, false, FR, JU>(p);
    if (p.done.count) {
        const unsigned long long total = LIST ? (*p.list_in_count + 31u) / 32u : 0u;
        done_signal(p.done,
                    (unsigned long long)p.tile_base + p.tile_limit >= total ? 3 : 1);
    }
}

// One cooperative launch: block 0 produces the reference orbit (all its
// threads), block 1 finishes its entries, every other block iterates pixels
// (FP32 pass) as soon as the entries they need are finished.  Pixel work per
// orbit step is larger than the producer's, so the orbit's serial time hides
// behind the pixels.  Cooperative launch guarantees the blocks are
// co-resident; every wait is bounded and raises orbit_error on timeout.
template <bool WANT_MAG>
__global__ void __launch_bounds__(256, 5) perturb_fused_kernel(OrbitLaunch o, PerturbLaunch p)
{
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0)
            *(volatile int*)p.producer_sm = (int)smid + 1;
        OrbitProgress g{p.raw_len, p.fin_len, p.orbit_done, p.orbit_error};
        orbit_produce(o, &g);
        return;
    }
    if (blockIdx.x == 1) {
        OrbitProgress g{p.raw_len, p.fin_len, p.orbit_done, p.orbit_error};
        orbit_finisher(o, g);
        return;
    }
    // The producer's latency-bound warps need their SM's issue slots: pixel
    // blocks placed on that SM leave at once (1/152 of the pixel capacity).
    __shared__ int s_leave;
    if (threadIdx.x == 0) {
        int sm = 0, spins = 0;
        while ((sm = *(volatile const int*)p.producer_sm) == 0 && ++spins < p.spin_limit)
            __nanosleep(64);
        s_leave = (sm == (int)smid + 1);
    }
    __syncthreads();
    if (s_leave)
        return;
    pixel_tiles<float, WANT_MAG, false, true, MDZ_MANDELBROT>(p);
}

// ---- serving: one step of the FP32 pass over a mixed work queue ----

// 32 bytes of resumable state per pixel (two uint4).  |z|^2 at escape is
// only read from a finished run, so an unfinished one keeps the error
// bound of the folded formulas in its place.
__device__ __forceinline__ void store_run(const PixRun<float>& r, uint4* sp)
{
    sp[0] = make_uint4(__float_as_uint(r.st.tr), __float_as_uint(r.st.ti), (unsigned)r.st.e,
                       (unsigned)r.m);
    sp[1] = make_uint4(r.wz, __float_as_uint(r.lost), __float_as_uint(r.st.e2), r.rebases);
}

__device__ __forceinline__ void load_run(PixRun<float>& r, const uint4* sp, double dcm_r,
                                         double dcm_i, int dce, float ke)
{
    const uint4 a = sp[0], b = sp[1];
    r.st.tr = __uint_as_float(a.x);
    r.st.ti = __uint_as_float(a.y);
    r.st.e = (int)a.z;
    r.m = (int)a.w;
    r.wz = b.x;
    r.lost = __uint_as_float(b.y);
    r.st.e2 = __uint_as_float(b.z);
    r.mag = 0.f;
    r.rebases = b.w;
    r.st.ke = ke;
    refresh_scale(r.st, (float)dcm_r, (float)dcm_i, dce);
}

// Warp-aggregated append of the lanes with `want` set to a queue.
__device__ __forceinline__ void queue_append(bool want, unsigned value, unsigned* q,
                                             unsigned* count)
{
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    if (!mask)
        return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane == leader)
        base = atomicAdd(count, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (want)
        q[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

// Lanes with `done` set subtract one each from remaining[slot], one atomic
// per distinct slot in the warp.
__device__ __forceinline__ void retire_pixels(bool done, int slot, unsigned* remaining)
{
    const unsigned mask = __ballot_sync(0xffffffffu, done);
    if (!done)
        return;
    const unsigned grp = __match_any_sync(mask, slot);
    if ((int)(threadIdx.x & 31) == __ffs(grp) - 1)
        atomicSub(remaining + slot, (unsigned)__popc(grp));
}

// Folded formulas carry the error estimate: 4 blocks per SM leave them 64
// registers (5 would spill).
template <int FR>
__global__ void __launch_bounds__(256, FR == MDZ_MANDELBROT ? 5 : 4)
    serve_perturb_kernel(ServeDev* __restrict__ d)
{
    // class = formula: 0 Mandelbrot, 1 burning ship, 2 celtic
    constexpr int cls = FR;
    if (serve_block_leaves(d, cls))
        return;
    const unsigned cur = d->ctl.cur;
    const unsigned n = d->status.qcount[cls][cur];
    const ServeClassTimer timer(d, cls, cur, n);
    const unsigned* qin = d->queue[cls][cur];
    unsigned* qout = d->queue[cls][cur ^ 1u];
    unsigned* qout_count = &d->status.qcount[cls][cur ^ 1u];
    const unsigned long long cancel = d->ctl.cancel;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned base = 0;
        if (lane == 0)
            base = atomicAdd(&d->qpull[cls], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const unsigned i = base + lane;
        const bool valid = i < n;
        const unsigned e = valid ? qin[i] : 0u;
        const int slot = (int)(e >> kEntrySlotShift);
        const unsigned pix = e & kEntryPixelMask;
        bool done = false, again = false;
        if (valid) {
            if ((cancel >> slot) & 1ull) {
                done = true;
            } else {
                const ServeReq& rq = d->req[slot];
                const PerturbLaunch& p = rq.pl;
                const int line = (int)(pix / (unsigned)p.W);
                const int ix = (int)(pix - (unsigned)line * (unsigned)p.W);
                const double dcm_r = (double)(2 * ix - p.W) * p.hs_m;
                const double dcm_i = (double)(p.H - 2 * line) * p.hs_m;
                uint4* sp = rq.state + (size_t)pix * 2u;
                PixRun<float> r;
                if (e & kEntryFresh)
                    pixel_start(r, dcm_r, dcm_i, p.hs_e, fold_ke<float>(p));
                else
                    load_run(r, sp, dcm_r, dcm_i, p.hs_e, fold_ke<float>(p));
                const uint32_t last = r.wz + d->ctl.budget[slot] - 1u;
                uint32_t count = 0;
                if (perturb_run<float, kOrbitSnapshot, FR>(p, r, dcm_r, dcm_i, p.hs_e, last, count,
                                                       nullptr, orbit_snapshot(p)) == 1) {
                    p.out[pix] = (int32_t)count;
                    if (p.mag)
                        p.mag[pix] = r.mag;
                    if (r.lost > p.lost_limit && p.flag_out)
                        p.flag_out[atomicAdd(p.flag_out_count, 1u)] = pix;
                    if (r.rebases)
                        atomicAdd(p.rebases, (unsigned long long)r.rebases);
                    done = true;
                } else {
                    store_run(r, sp);
                    again = true;
                }
            }
        }
        queue_append(again, e & ~kEntryFresh, qout, qout_count);
        retire_pixels(done, slot, d->status.remaining);
    }
}

// ---- streamed orbit: pixels start while the orbit is being iterated ----

// Block 0: the producer (the lean form for the orbit's digit count); block
// 1: the finisher (batches of blockDim.x entries).  Launched cooperatively
// (both blocks resident at once: the finisher waits, bounded, on the
// producer's progress).
template <int MAXP, int NSLOT>
__global__ void __launch_bounds__(1024) orbit_stream_kernel(OrbitLaunch o, OrbitProgress g,
                                                            int* producer_sm, DoneSignal done)
{
    if (blockIdx.x == 0) {
        unsigned smid = 0;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        if (threadIdx.x == 0) {
            if (o.sm_busy)
                atomicAdd(o.sm_busy + smid % (unsigned)o.sm_words, 1);
            *(volatile int*)producer_sm = (int)smid + 1;
        }
        orbit_produce_lean<MAXP, NSLOT>(o, &g);
        if (threadIdx.x == 0) {
            *(volatile int*)producer_sm = 0;
            if (o.sm_busy)
                atomicSub(o.sm_busy + smid % (unsigned)o.sm_words, 1);
        }
    } else {
        orbit_finisher(o, g);
    }
    if (done.count)
        done_signal(done, *(volatile int*)g.error ? 2 : 1);
}

// One step of the FP32 pass of one frame over a compacted pixel queue:
// entries in[0 .. n) (in == nullptr: entry i is pixel i, fresh), every pixel
// iterates at most `budget` iterations or until it needs an orbit entry not
// finished yet; unfinished pixels are appended to out.
struct FrameStep {
    const unsigned* in;
    unsigned n;
    unsigned* out;
    unsigned* out_count;
    unsigned* pull;
    unsigned* workers;   // blocks working this launch
    uint4* state;        // 32 bytes per pixel
    unsigned budget;
};

template <bool WANT_MAG, int FR>
__global__ void __launch_bounds__(256, FR == MDZ_MANDELBROT ? 5 : 4)
    perturb_step_kernel(PerturbLaunch p, FrameStep q)
{
    // leave the orbit producer's SM to it, unless no other block works yet
    // (a working block pulls until the queue is empty)
    __shared__ int s_leave;
    if (threadIdx.x == 0) {
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        const bool producer_here = *(volatile const int*)p.producer_sm == (int)smid + 1;
        s_leave = producer_here && *(volatile const unsigned*)q.workers > 0u;
        if (!s_leave)
            atomicAdd(q.workers, 1u);
    }
    __syncthreads();
    if (s_leave)
        return;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned base = 0;
        if (lane == 0)
            base = atomicAdd(q.pull, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= q.n)
            break;
        const unsigned i = base + lane;
        const bool valid = i < q.n;
        const unsigned e = valid ? (q.in ? q.in[i] : (i | kEntryFresh)) : 0u;
        const unsigned pix = e & kEntryPixelMask;
        bool again = false;
        unsigned long long its = 0;
        unsigned reb = 0;
        if (valid) {
            const int line = (int)(pix / (unsigned)p.W);
            const int ix = (int)(pix - (unsigned)line * (unsigned)p.W);
            const double dcm_r = (double)(2 * ix - p.W) * p.hs_m;
            const double dcm_i = (double)(p.H - 2 * (p.row0 + line)) * p.hs_m;
            uint4* sp = q.state + (size_t)pix * 2u;
            PixRun<float> r;
            if (e & kEntryFresh)
                pixel_start(r, dcm_r, dcm_i, p.hs_e, fold_ke<float>(p));
            else
                load_run(r, sp, dcm_r, dcm_i, p.hs_e, fold_ke<float>(p));
            const uint32_t last = r.wz + q.budget - 1u;
            uint32_t count = 0;
            if (perturb_run<float, kOrbitSnapshot, FR>(p, r, dcm_r, dcm_i, p.hs_e, last, count,
                                                   nullptr, orbit_snapshot(p)) == 1) {
                p.out[pix] = (int32_t)count;
                if (WANT_MAG)
                    p.mag[pix] = r.mag;
                if (r.lost > p.lost_limit && p.flag_out)
                    p.flag_out[atomicAdd(p.flag_out_count, 1u)] = pix;
                else
                    its = count ? count : p.depth;
                reb = r.rebases;
            } else {
                store_run(r, sp);
                again = true;
            }
        }
        queue_append(again, pix, q.out, q.out_count);
        its = warp_sum_u64(its);
        const unsigned long long rb = warp_sum_u64((unsigned long long)reb);
        if (lane == 0) {
            if (its)
                atomicAdd(&p.sync->iter_sum, its);
            if (rb)
                atomicAdd(p.rebases, rb);
        }
    }
}

__global__ void frame_step_reset_kernel(unsigned* counters)
{
    counters[0] = 0u;   // pull
    counters[1] = 0u;   // out count
    counters[2] = 0u;   // workers
}

__global__ void serve_enqueue_kernel(ServeDev* d, int cls, int q, int slot, unsigned npix)
{
    unsigned* queue = d->queue[cls][q];
    const unsigned base = d->status.qcount[cls][q];
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x)
        queue[base + i] = serve_entry(slot, true, i);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        d->status.remaining[slot] = npix;
}

__global__ void serve_enqueue_count_kernel(ServeDev* d, int cls, int q, unsigned npix)
{
    d->status.qcount[cls][q] += npix;
}

__global__ void serve_step_end_kernel(ServeDev* d)
{
    const unsigned cur = d->ctl.cur;
    for (int c = threadIdx.x; c < kServeClasses; c += blockDim.x) {
        d->status.qcount[c][cur] = 0u;
        d->qpull[c] = 0u;
        d->qworkers[c] = 0u;
        d->status.tk[cur ^ 1u][c][0] = ~0ull;   // the next step's time span
        d->status.tk[cur ^ 1u][c][1] = 0ull;
    }
    for (int slot = threadIdx.x; slot < kServeSlots; slot += blockDim.x) {
        const unsigned* fc = d->req[slot].pl.flag_out_count;
        d->status.flagged[slot] = fc ? *fc : 0u;
    }
    if (threadIdx.x == 0)
        d->status.tstep[cur][1] = ServeClassTimer::now();
}

__global__ void serve_step_begin_kernel(ServeDev* d)
{
    d->status.tstep[d->ctl.cur][0] = ServeClassTimer::now();
}

}  // namespace

int launch_serve_perturb(ServeDev* d, int formula, int num_sms, cudaStream_t s)
{
    const void* fn = formula == MDZ_BURNING_SHIP         ? (const void*)serve_perturb_kernel<1>
                     : formula == MDZ_GENERALIZED_CELTIC ? (const void*)serve_perturb_kernel<2>
                                                         : (const void*)serve_perturb_kernel<0>;
    static int bps = 0;
    if (!bps) {
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, 256, 0));
        if (bps < 1)
            bps = 1;
    }
    const unsigned grid = (unsigned)(num_sms * bps);
    if (formula == MDZ_BURNING_SHIP)
        serve_perturb_kernel<1><<<grid, 256, 0, s>>>(d);
    else if (formula == MDZ_GENERALIZED_CELTIC)
        serve_perturb_kernel<2><<<grid, 256, 0, s>>>(d);
    else
        serve_perturb_kernel<0><<<grid, 256, 0, s>>>(d);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

int launch_serve_enqueue(ServeDev* d, int cls, int q, int slot, unsigned npix, cudaStream_t s)
{
    const unsigned blocks = npix ? (npix + 255u) / 256u : 1u;
    serve_enqueue_kernel<<<blocks < 1024u ? blocks : 1024u, 256, 0, s>>>(d, cls, q, slot, npix);
    MDZ_CUDA_TRY(cudaGetLastError());
    serve_enqueue_count_kernel<<<1, 1, 0, s>>>(d, cls, q, npix);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

int launch_serve_step_end(ServeDev* d, cudaStream_t s)
{
    serve_step_end_kernel<<<1, 32, 0, s>>>(d);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

int launch_serve_step_begin(ServeDev* d, cudaStream_t s)
{
    serve_step_begin_kernel<<<1, 1, 0, s>>>(d);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

int launch_orbit_stream(const OrbitLaunch& o, int* progress, cudaStream_t s, DoneSignal done)
{
    if (o.limbs < 5 || o.limbs > kMaxOrbitLimbs) {
        set_error("orbit: %d limbs outside [5, %d]", o.limbs, kMaxOrbitLimbs);
        return MDZGPU_ERR_UNSUPPORTED;
    }
    OrbitLaunch oo = o;
    OrbitProgress g{progress + 1, progress + 2, progress + 3, progress + 4};
    int* producer_sm = progress + 5;
    void* args[] = {&oo, &g, &producer_sm, &done};
    const void* fn = nullptr;
#define MDZ_CASE(lmax, mp, ns)                                      \
    if (!fn && o.limbs <= lmax)                                     \
        fn = (const void*)orbit_stream_kernel<mp, ns>;
    MDZ_ORBIT_LEAN_CASES(MDZ_CASE)
#undef MDZ_CASE
    MDZ_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(2), dim3(orbit_lean_threads(o.limbs)),
                                             args, 0, s));
    return MDZGPU_OK;
}

int launch_perturb_step(int num_sms, const PerturbLaunch& p, const unsigned* in, unsigned n,
                        unsigned* out, unsigned* counters, uint4* state, unsigned budget,
                        cudaStream_t s, cudaEvent_t before, cudaEvent_t after)
{
    const bool mag = p.mag != nullptr;
    const int fr = p.fractal == MDZ_BURNING_SHIP ? 1 : p.fractal == MDZ_GENERALIZED_CELTIC ? 2 : 0;
    const void* fns[2][3] = {{(const void*)perturb_step_kernel<false, 0>,
                              (const void*)perturb_step_kernel<false, 1>,
                              (const void*)perturb_step_kernel<false, 2>},
                             {(const void*)perturb_step_kernel<true, 0>,
                              (const void*)perturb_step_kernel<true, 1>,
                              (const void*)perturb_step_kernel<true, 2>}};
    const void* fn = fns[mag ? 1 : 0][fr];
    static int bps[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int& b = bps[mag ? 1 : 0][fr];
    if (!b) {
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, 256, 0));
        if (b < 1)
            b = 1;
    }
    long grid = (long)num_sms * b;
    const long needed = ((long)n + 255) / 256;
    if (grid > needed)
        grid = needed;
    if (grid < 1)
        grid = 1;
    frame_step_reset_kernel<<<1, 1, 0, s>>>(counters);
    MDZ_CUDA_TRY(cudaGetLastError());
    FrameStep q{in, n, out, counters + 1, counters, counters + 2, state, budget};
    if (before)
        MDZ_CUDA_TRY(cudaEventRecord(before, s));
    void* args[] = {(void*)&p, (void*)&q};
    MDZ_CUDA_TRY(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(256), args, 0, s));
    MDZ_CUDA_TRY(cudaGetLastError());
    if (after)
        MDZ_CUDA_TRY(cudaEventRecord(after, s));
    return MDZGPU_OK;
}

int launch_orbit(const OrbitLaunch& p, cudaStream_t s)
{
    if (p.limbs < 5 || p.limbs > kMaxOrbitLimbs) {
        set_error("orbit: %d limbs outside [5, %d]", p.limbs, kMaxOrbitLimbs);
        return MDZGPU_ERR_UNSUPPORTED;
    }
    bool launched = false;
#define MDZ_CASE(lmax, mp, ns)                                                   \
    if (!launched && p.limbs <= lmax) {                                          \
        orbit_kernel_lean<mp, ns><<<1, orbit_lean_threads(p.limbs), 0, s>>>(p); \
        launched = true;                                                         \
    }
    MDZ_ORBIT_LEAN_CASES(MDZ_CASE)
#undef MDZ_CASE
    MDZ_CUDA_TRY(cudaGetLastError());
    orbit_finish_kernel<<<(p.max_k + 1 + 127) / 128, 128, 0, s>>>(p);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

template <class T, bool WANT_MAG, bool LIST, int FR, bool JU = false>
int pass_blocks_per_sm(int* out)
{
    static int bps = 0;
    if (!bps) {
        int b = 0;
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, perturb_kernel<T, WANT_MAG, LIST, FR, JU>, 256, 0));
        bps = b < 1 ? 1 : b;
    }
    *out = bps;
    return MDZGPU_OK;
}

template <class T, bool WANT_MAG, bool LIST, int FR, bool JU>
int launch_pass_fr(mdzgpu_ctx* ctx, const PerturbLaunch& p, cudaStream_t s, long work_items)
{
    int bps = 1;
    if (int rc = pass_blocks_per_sm<T, WANT_MAG, LIST, FR, JU>(&bps))
        return rc;
    long grid = (long)ctx->num_sms * bps;
    const long blocks_needed = (work_items + 7) / 8;
    if (grid > blocks_needed)
        grid = blocks_needed;
    if (grid < 1)
        grid = 1;
    perturb_kernel<T, WANT_MAG, LIST, FR, JU><<<(unsigned)grid, 256, 0, s>>>(p);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

template <class T, bool WANT_MAG, bool LIST, bool JU>
int launch_pass_ju(mdzgpu_ctx* ctx, const PerturbLaunch& p, cudaStream_t s, long work_items)
{
    if (p.fractal == MDZ_VARIANT && !JU)
        return launch_pass_fr<T, WANT_MAG, LIST, MDZ_VARIANT, false>(ctx, p, s, work_items);
    if (p.fractal == MDZ_BURNING_SHIP)
        return launch_pass_fr<T, WANT_MAG, LIST, 1, JU>(ctx, p, s, work_items);
    if (p.fractal == MDZ_GENERALIZED_CELTIC)
        return launch_pass_fr<T, WANT_MAG, LIST, 2, JU>(ctx, p, s, work_items);
    return launch_pass_fr<T, WANT_MAG, LIST, 0, JU>(ctx, p, s, work_items);
}

template <class T, bool WANT_MAG, bool LIST>
int launch_pass(mdzgpu_ctx* ctx, const PerturbLaunch& p, cudaStream_t s, long work_items)
{
    return p.julia ? launch_pass_ju<T, WANT_MAG, LIST, true>(ctx, p, s, work_items)
                   : launch_pass_ju<T, WANT_MAG, LIST, false>(ctx, p, s, work_items);
}

template <int FR>
int preload_fr()
{
    int b = 0, rc = MDZGPU_OK;
    if (!rc)
        rc = pass_blocks_per_sm<float, false, false, FR>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<float, true, false, FR>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<double, false, true, FR>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<double, true, true, FR>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<float, false, false, FR, true>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<float, true, false, FR, true>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<double, false, true, FR, true>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<double, true, true, FR, true>(&b);
    cudaFuncAttributes a;
    if (!rc && (cudaFuncGetAttributes(&a, perturb_step_kernel<false, FR>) != cudaSuccess
                || cudaFuncGetAttributes(&a, perturb_step_kernel<true, FR>) != cudaSuccess
                || cudaFuncGetAttributes(&a, serve_perturb_kernel<FR>) != cudaSuccess))
        rc = MDZGPU_ERR_CUDA;
    return rc;
}

int preload_perturb_kernels()
{
    int b = 0;
    int rc = pass_blocks_per_sm<float, false, false, MDZ_VARIANT>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<float, true, false, MDZ_VARIANT>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<double, false, true, MDZ_VARIANT>(&b);
    if (!rc)
        rc = pass_blocks_per_sm<double, true, true, MDZ_VARIANT>(&b);
    if (!rc)
        rc = preload_fr<MDZ_MANDELBROT>();
    if (!rc)
        rc = preload_fr<MDZ_BURNING_SHIP>();
    if (!rc)
        rc = preload_fr<MDZ_GENERALIZED_CELTIC>();
    cudaFuncAttributes a;
#define MDZ_CASE(lmax, mp, ns)                                                        \
    if (!rc && (cudaFuncGetAttributes(&a, orbit_stream_kernel<mp, ns>) != cudaSuccess \
                || cudaFuncGetAttributes(&a, orbit_kernel_lean<mp, ns>) != cudaSuccess)) \
        rc = MDZGPU_ERR_CUDA;
    MDZ_ORBIT_LEAN_CASES(MDZ_CASE)
#undef MDZ_CASE
    if (!rc && (cudaFuncGetAttributes(&a, orbit_finish_kernel) != cudaSuccess
                || cudaFuncGetAttributes(&a, frame_step_reset_kernel) != cudaSuccess
                || cudaFuncGetAttributes(&a, serve_enqueue_kernel) != cudaSuccess
                || cudaFuncGetAttributes(&a, serve_enqueue_count_kernel) != cudaSuccess
                || cudaFuncGetAttributes(&a, serve_step_begin_kernel) != cudaSuccess
                || cudaFuncGetAttributes(&a, serve_step_end_kernel) != cudaSuccess))
        rc = MDZGPU_ERR_CUDA;
    if (rc == MDZGPU_ERR_CUDA)
        set_error("perturbation: loading the kernels failed");
    return rc;
}

int launch_perturb(mdzgpu_ctx* ctx, const PerturbLaunch& p, cudaStream_t s, int pass)
{
    const bool mag = p.mag != nullptr;
    if (pass == 0) {
        const long tiles = (long)((p.W + kTileW - 1) / kTileW) * ((p.nrows + kTileH - 1) / kTileH);
        return mag ? launch_pass<float, true, false>(ctx, p, s, tiles)
                   : launch_pass<float, false, false>(ctx, p, s, tiles);
    }
    // list pass: sized for the worst case, exits at once on an empty list
    const long chunks = ((long)p.W * p.nrows + 31) / 32;
    return mag ? launch_pass<double, true, true>(ctx, p, s, chunks)
               : launch_pass<double, false, true>(ctx, p, s, chunks);
}

int launch_fused(mdzgpu_ctx* ctx, const OrbitLaunch& o, const PerturbLaunch& p, cudaStream_t s)
{
    if (o.limbs < 5 || o.limbs > kMaxOrbitLimbs) {
        set_error("orbit: %d limbs outside [5, %d]", o.limbs, kMaxOrbitLimbs);
        return MDZGPU_ERR_UNSUPPORTED;
    }
    const bool mag = p.mag != nullptr;
    const void* fn = mag ? (const void*)perturb_fused_kernel<true>
                         : (const void*)perturb_fused_kernel<false>;
    static int bps[2] = {0, 0};
    int& b = bps[mag ? 1 : 0];
    if (!b) {
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, 256, 0));
        if (b < 1)
            b = 1;
    }
    int coop = 0;
    MDZ_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
    if (!coop) {
        set_error("device lacks cooperative launch");
        return MDZGPU_ERR_UNSUPPORTED;
    }
    const long tiles = (long)((p.W + kTileW - 1) / kTileW) * ((p.nrows + kTileH - 1) / kTileH);
    long grid = (long)ctx->num_sms * b;          // all co-resident
    const long needed = 2 + (tiles + 7) / 8;
    if (grid > needed)
        grid = needed;
    if (grid < 3)
        grid = 3;
    if (grid > (long)ctx->num_sms * b) {
        set_error("fused launch needs %ld co-resident blocks", grid);
        return MDZGPU_ERR_UNSUPPORTED;
    }
    OrbitLaunch oo = o;
    PerturbLaunch pp = p;
    void* args[] = {&oo, &pp};
    MDZ_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3((unsigned)grid), dim3(256), args, 0, s));
    return MDZGPU_OK;
}

int orbit_max_limbs()
{
    return kMaxOrbitLimbs;
}

}  // namespace mdz
