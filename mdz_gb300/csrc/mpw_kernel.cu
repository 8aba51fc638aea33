// Multi-limb fixed-point escape-time kernel for precisions beyond one
// thread's registers: a group of G lanes iterates one pixel.
//
// Same reference loops and count semantics as mp_kernel.cu (MDZ's MPFR /
// GMP paths, src/frac_mandel.c:25-82 and siblings; pixel coordinates of
// src/fractal.c:159-192 / :299-332 computed on the host).  The number
// format is the one of fixed_point.cuh -- two's complement, F = 64 NL - 8
// fractional bits -- held as NL = G Q 64-bit limbs, lane l of the group
// owning limbs [l Q, l Q + Q).
//
//  * Additions: each lane adds its Q limbs with a 64-bit carry chain
//    (add.cc.u64 / addc.u64); the carries between lanes are resolved with
//    two ballots (generate / propagate) and one integer addition -- the
//    carry-lookahead identity C = (g + (g | p) + c0) ^ p over the group's
//    lanes.
//  * Products (one general, two squares per iteration) are truncated like
//    the one-thread kernel (partial products with i + j < NL - 2 skipped).
//    The operands go to shared memory; lane l forms the 192-bit sums of the
//    columns c = NL - 2 + l + G t (interleaved, so every lane gets short
//    and long columns) with mad.lo.cc.u64 / madc.hi.cc.u64; the three
//    64-bit parts of every column go back to shared memory shifted by 0, 1
//    and 2 limbs and are added as distributed numbers (lane carries as
//    above); the result is the window F .. F + 64 NL of that sum.
//
// The four (G = 8) or one (G = 32) pixels of a warp run in lock step: a
// group whose pixel finishes writes its count and takes the next pixel
// (or idles) while the others go on.  Every shuffle and ballot is a
// full-warp operation, so each one is executed by all 32 lanes at the same
// point of the loop -- never inside a branch or a short-circuit that can
// differ between the groups (that would leave lanes named in the mask out
// of the operation).
#include "internal.h"

namespace mdz {
namespace {

constexpr int kMpwBlock = 128;

__device__ __forceinline__ unsigned long long warp_sum_its(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ uint64_t mad_lo_cc(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t r;
    asm volatile("mad.lo.cc.u64 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ uint64_t madc_hi_cc(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t r;
    asm volatile("madc.hi.cc.u64 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ uint64_t addc_0(uint64_t a)
{
    uint64_t r;
    asm volatile("addc.u64 %0, %1, 0;" : "=l"(r) : "l"(a));
    return r;
}

template <int G, int Q>
struct Mpw {
    static constexpr int NL = G * Q;          // limbs per number
    static constexpr int QP = Q + 1;          // limbs per lane of the column sums
    static constexpr int NP = G * QP;         // >= NL + 3 positions (G >= 4)
    static_assert(G >= 4 && G <= 32 && (32 % G) == 0, "group of 4..32 lanes");

    // shared memory of one group
    struct Smem {
        uint64_t a[NL], b[NL];               // operands
        uint64_t t0[NP], t1[NP], t2[NP];     // column-sum parts; position p = column NL-2+p
    };

    int pl;          // lane within the group
    int gbase;       // first lane of the group in the warp
    Smem* sm;

    __device__ __forceinline__ Mpw(Smem* s)
    {
        const int lane = threadIdx.x & 31;
        pl = lane % G;
        gbase = lane - pl;
        sm = s;
    }

    // carry into this lane of a group-wide addition: gen = this lane's
    // carry out, prop = its sum is all ones, c0 = carry into lane 0
    __device__ __forceinline__ uint32_t lane_carry(bool gen, bool prop, uint32_t c0) const
    {
        const uint32_t gm32 = __ballot_sync(0xffffffffu, gen);
        const uint32_t pm32 = __ballot_sync(0xffffffffu, prop);
        const uint64_t msk = G == 32 ? 0xffffffffull : ((1ull << G) - 1ull);
        const uint64_t gm = ((uint64_t)gm32 >> gbase) & msk;
        const uint64_t pm = ((uint64_t)pm32 >> gbase) & msk;
        const uint64_t c = (gm + (gm | pm) + (uint64_t)c0) ^ pm;
        return (uint32_t)(c >> pl) & 1u;
    }

    // r = x + y + c0 (c0 into the group's lowest limb), K limbs per lane
    template <int K>
    __device__ __forceinline__ void add(const uint64_t (&x)[K], const uint64_t (&y)[K],
                                        uint32_t c0, uint64_t (&r)[K]) const
    {
        uint64_t s[K];
        uint64_t cout;
        asm volatile("add.cc.u64 %0, %1, %2;" : "=l"(s[0]) : "l"(x[0]), "l"(y[0]));
#pragma unroll
        for (int k = 1; k < K; ++k)
            asm volatile("addc.cc.u64 %0, %1, %2;" : "=l"(s[k]) : "l"(x[k]), "l"(y[k]));
        asm volatile("addc.u64 %0, 0, 0;" : "=l"(cout));
        uint64_t all = s[0];
#pragma unroll
        for (int k = 1; k < K; ++k)
            all &= s[k];
        const uint32_t cin = lane_carry(cout != 0ull, all == ~0ull, c0);
        asm volatile("add.cc.u64 %0, %1, %2;" : "=l"(r[0]) : "l"(s[0]), "l"((uint64_t)cin));
#pragma unroll
        for (int k = 1; k < K; ++k)
            asm volatile("addc.cc.u64 %0, %1, 0;" : "=l"(r[k]) : "l"(s[k]));
    }

    // r = c + (x ^ m) + (m & 1): c + x when m == 0, c - x when m == ~0
    __device__ __forceinline__ void add_signed(const uint64_t (&c)[Q], const uint64_t (&x)[Q],
                                               uint64_t m, uint64_t (&r)[Q]) const
    {
        uint64_t xm[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k)
            xm[k] = x[k] ^ m;
        add<Q>(c, xm, (uint32_t)(m & 1ull), r);
    }

    // r = a - b
    __device__ __forceinline__ void sub(const uint64_t (&a)[Q], const uint64_t (&b)[Q],
                                        uint64_t (&r)[Q]) const
    {
        uint64_t nb[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k)
            nb[k] = ~b[k];
        add<Q>(a, nb, 1u, r);
    }

    // the group's top limb (lane G-1's last), on every lane of the group
    __device__ __forceinline__ uint64_t top(const uint64_t (&x)[Q]) const
    {
        return __shfl_sync(0xffffffffu, x[Q - 1], gbase + G - 1);
    }

    // in place |x|; returns the sign mask (0 or ~0) of the input
    __device__ __forceinline__ uint64_t abs_inplace(uint64_t (&x)[Q]) const
    {
        const uint64_t m = (uint64_t)((int64_t)top(x) >> 63);
        uint64_t xm[Q], z[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            xm[k] = x[k] ^ m;
            z[k] = 0ull;
        }
        add<Q>(xm, z, (uint32_t)(m & 1ull), x);
        return m;
    }

    // |x| >= 8: the value has escaped and squaring it could overflow
    __device__ __forceinline__ bool big(const uint64_t (&x)[Q]) const
    {
        const int64_t t = (int64_t)top(x);
        return t >= 0x0800000000000000ll || t < -0x0800000000000000ll;
    }

    // a + b > 4 for non-negative a, b (< 64 each)
    __device__ __forceinline__ bool sum_gt4(const uint64_t (&a)[Q], const uint64_t (&b)[Q]) const
    {
        uint64_t s[Q];
        add<Q>(a, b, 0u, s);
        uint64_t low = 0ull;
#pragma unroll
        for (int k = 0; k < Q; ++k)
            if (pl != G - 1 || k < Q - 1)
                low |= s[k];
        const uint32_t nz = __ballot_sync(0xffffffffu, low != 0ull);
        const bool low_nz = ((nz >> gbase) & (G == 32 ? 0xffffffffu : ((1u << G) - 1u))) != 0u;
        const uint64_t t = top(s);
        return t > 0x0400000000000000ull || (t == 0x0400000000000000ull && low_nz);
    }

    // top two limbs as a float (|value| < 128)
    __device__ __forceinline__ float top_float(const uint64_t (&x)[Q]) const
    {
        const uint64_t t = top(x);
        const uint64_t n = __shfl_sync(0xffffffffu, Q >= 2 ? x[Q - 2] : x[Q - 1],
                                       Q >= 2 ? gbase + G - 1 : gbase + G - 2);
        return (float)(int64_t)t * 1.3877788e-17f /* 2^-56 */
               + (float)n * 7.5231638e-37f /* 2^-120 */;
    }

    // r = floor(a b / 2^(F - SQ)) restricted to NL limbs (truncated
    // product; SQ = 1 doubles it), a and b magnitudes; SQUARE: b == a
    template <bool SQUARE, int SQ>
    __device__ __forceinline__ void mul(const uint64_t (&a)[Q], const uint64_t (&b)[Q],
                                        uint64_t (&r)[Q]) const
    {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            sm->a[pl * Q + k] = a[k];
            if (!SQUARE)
                sm->b[pl * Q + k] = b[k];
        }
        // positions no column writes (see below) start at zero
        if (pl == 0) {
            sm->t1[0] = 0ull;
            sm->t2[0] = 0ull;
            sm->t2[1] = 0ull;
        }
#pragma unroll
        for (int p = NL + 1 + pl; p < NP; p += G) {
            sm->t0[p] = 0ull;
            if (p >= NL + 2)
                sm->t1[p] = 0ull;
            if (p >= NL + 3)
                sm->t2[p] = 0ull;
        }
        __syncwarp();
        const uint64_t* A = sm->a;
        const uint64_t* B = SQUARE ? sm->a : sm->b;
        constexpr int NC = NL + 1;                       // columns NL-2 .. 2NL-2
        constexpr int T = (NC + G - 1) / G;
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int p = pl + G * t;
            if (p < NC) {
                const int c = NL - 2 + p;
                const int ilo = c - (NL - 1) > 0 ? c - (NL - 1) : 0;
                uint64_t s0 = 0ull, s1 = 0ull, s2 = 0ull;
                if (SQUARE) {
                    // off-diagonal terms i < j once, doubled, plus the diagonal
                    const int ihi = (c - 1) >> 1;
                    for (int i = ilo; i <= ihi; ++i) {
                        const uint64_t x = A[i], y = A[c - i];
                        s0 = mad_lo_cc(x, y, s0);
                        s1 = madc_hi_cc(x, y, s1);
                        s2 = addc_0(s2);
                    }
                    s2 = (s2 << 1) | (s1 >> 63);
                    s1 = (s1 << 1) | (s0 >> 63);
                    s0 <<= 1;
                    if (!(c & 1)) {
                        const uint64_t h = A[c >> 1];
                        s0 = mad_lo_cc(h, h, s0);
                        s1 = madc_hi_cc(h, h, s1);
                        s2 = addc_0(s2);
                    }
                } else {
                    const int ihi = c < NL - 1 ? c : NL - 1;
                    for (int i = ilo; i <= ihi; ++i) {
                        const uint64_t x = A[i], y = B[c - i];
                        s0 = mad_lo_cc(x, y, s0);
                        s1 = madc_hi_cc(x, y, s1);
                        s2 = addc_0(s2);
                    }
                }
                sm->t0[p] = s0;
                sm->t1[p + 1] = s1;
                sm->t2[p + 2] = s2;
            }
        }
        __syncwarp();
        uint64_t u0[QP], u1[QP], u2[QP];
#pragma unroll
        for (int k = 0; k < QP; ++k) {
            u0[k] = sm->t0[pl * QP + k];
            u1[k] = sm->t1[pl * QP + k];
            u2[k] = sm->t2[pl * QP + k];
        }
        add<QP>(u0, u1, 0u, u0);
        add<QP>(u0, u2, 0u, u0);
        __syncwarp();
#pragma unroll
        for (int k = 0; k < QP; ++k)
            sm->t0[pl * QP + k] = u0[k];
        __syncwarp();
        // r[k] = bits F - SQ + 64 k .. of the sum: position k + 1 holds bit F
        // at offset 56 (F = 64 NL - 8, position 1 = column NL - 1)
        constexpr int SH = 56 - SQ;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const int g = pl * Q + k;
            const uint64_t lo = sm->t0[g + 1], hi = sm->t0[g + 2];
            r[k] = (lo >> SH) | (hi << (64 - SH));
        }
        __syncwarp();
    }
};

template <int G, int Q, int FRACTAL, bool JULIA>
__global__ void __launch_bounds__(kMpwBlock) mpw_frame_kernel(MpLaunch p)
{
    using M = Mpw<G, Q>;
    constexpr int NL = M::NL;
    constexpr int N = 2 * NL;                      // 32-bit words of the host tables
    constexpr int GPB = kMpwBlock / G;             // groups per block
    __shared__ typename M::Smem smem[GPB];
    const int lane = threadIdx.x & 31;
    const int group = threadIdx.x / G;
    M mp(&smem[group]);
    const bool leader = mp.pl == 0;
    const unsigned list_n = p.list ? *p.list_count : 0u;
    const unsigned total = p.list ? list_n : (unsigned)p.W * (unsigned)p.nrows;
    // chunks of a list pass (tile_base / tile_limit) count 32 pixels a unit,
    // as the one-thread kernel's tiles do; pixels are taken in list or
    // row-major order
    const unsigned long long base = 32ull * p.tile_base;
    const unsigned long long limit =
        p.tile_limit == 0xffffffffu ? 0xffffffffffffffffull : 32ull * p.tile_limit;
    // group state
    uint64_t wre[Q], wim[Q], cre[Q], cim[Q], wre2[Q], wim2[Q];
    uint32_t wz = 0;
    unsigned pix = 0;
    bool active = false, fresh = false;
    unsigned long long its = 0;

    // takes the group's next pixel (all lanes call it; `need` per group)
    auto next_pixel = [&](bool need) {
        unsigned idx = 0xffffffffu;
        if (need && leader) {
            const unsigned t = (p.stop && *p.stop) ? 0xffffffffu
                                                    : atomicAdd(&p.sync->tile_counter, 1u);
            const unsigned long long i = base + t;
            idx = (t != 0xffffffffu && t < limit && i < total) ? (unsigned)i : 0xffffffffu;
        }
        idx = __shfl_sync(0xffffffffu, idx, mp.gbase);
        if (!need)
            return;
        active = idx != 0xffffffffu;
        if (!active)
            return;
        pix = p.list ? p.list[idx] : idx;
        const unsigned lrow = pix / (unsigned)p.W;
        const unsigned ix = pix - lrow * (unsigned)p.W;
        const uint64_t* xs = (const uint64_t*)(p.xs + (size_t)ix * N);
        const uint64_t* ys = (const uint64_t*)(p.ys + (size_t)lrow * N);
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            wre[k] = xs[mp.pl * Q + k];
            wim[k] = ys[mp.pl * Q + k];
            if (JULIA) {
                cre[k] = ((const uint64_t*)p.julia)[mp.pl * Q + k];
                cim[k] = ((const uint64_t*)(p.julia + N))[mp.pl * Q + k];
            } else {
                cre[k] = wre[k];
                cim[k] = wim[k];
            }
        }
        wz = 1;
        fresh = true;
    };
    auto finish = [&](uint32_t count, float mag) {
        if (leader) {
            p.out[pix] = (int32_t)count;
            if (p.mag)
                p.mag[pix] = mag;
            its += count ? count : p.depth;
            // progressive rows (the drop-in layer): a 4-row band is complete
            // when all its pixels are
            if (p.tile_rows_done && !p.list) {
                const unsigned band = (pix / (unsigned)p.W) / 4u;
                const unsigned rows = min(4u, (unsigned)p.nrows - 4u * band);
                if (p.band_flags)
                    __threadfence_system();
                const unsigned done = atomicAdd(&p.tile_rows_done[band], 1u) + 1u;
                if (done == rows * (unsigned)p.W && p.band_flags) {
                    __threadfence_system();
                    p.band_flags[band] = 1;
                }
            }
        }
    };

    next_pixel(true);
    for (;;) {
        if (!__any_sync(0xffffffffu, active))
            break;
        // |z_{wz-1}|^2 (escape test of the last iteration; none for z_0 = c)
        const uint64_t sre = mp.abs_inplace(wre);
        const uint64_t sim = mp.abs_inplace(wim);
        mp.template mul<true, 0>(wre, wre, wre2);
        mp.template mul<true, 0>(wim, wim, wim2);
        // every warp-wide step (the shuffles and ballots inside top, big,
        // sum_gt4, top_float) runs on all lanes, never under a condition
        // that differs between groups
        const bool gt4 = mp.sum_gt4(wim2, wre2);
        const float mag2 = mp.top_float(wim2) + mp.top_float(wre2);
        bool done = false;
        uint32_t count = 0;
        float mag = 0.f;
        if (active && !fresh && gt4) {
            done = true;
            count = wz - 1;
            mag = mag2;
        } else if (active && wz > p.depth) {
            done = true;
            count = 0;
            mag = mag2;
        }
        fresh = false;
        // iteration wz: wim = 2 wre wim + c_im (burning ship: 2 |wre wim| +
        // c_im); wre = wre2 - wim2 + c_re (celtic: |wre2 - wim2| + c_re)
        uint64_t t[Q], d[Q];
        mp.template mul<false, 1>(wre, wim, t);
        const uint64_t mt = (FRACTAL == MDZ_BURNING_SHIP) ? 0ull : (sre ^ sim);
        uint64_t nre[Q], nim[Q];
        mp.add_signed(cim, t, mt, nim);
        mp.sub(wre2, wim2, d);
        uint64_t md = 0ull;
        if (FRACTAL == MDZ_GENERALIZED_CELTIC || FRACTAL == MDZ_VARIANT) {
            const uint64_t sd = (uint64_t)((int64_t)mp.top(d) >> 63);
            if (FRACTAL == MDZ_GENERALIZED_CELTIC || (wz & 1u))
                md = sd;
        }
        mp.add_signed(cre, d, md, nre);
        const bool big_re = mp.big(nre);
        const bool big_im = mp.big(nim);
        const float fa = mp.top_float(nre), fb = mp.top_float(nim);
        if (active && !done && (big_re || big_im)) {
            done = true;
            count = wz;
            mag = fa * fa + fb * fb;
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            wre[k] = nre[k];
            wim[k] = nim[k];
        }
        ++wz;
        if (active && done)
            finish(count, mag);
        next_pixel(active && done);
    }
    its = warp_sum_its(its);
    if (lane == 0 && its)
        atomicAdd(&p.sync->iter_sum, its);
    if (p.done.count) {
        const bool end = p.tile_limit == 0xffffffffu || base + limit >= (unsigned long long)total;
        done_signal(p.done, end ? 3 : 1);
    }
}

template <int G, int Q, int FRACTAL, bool JULIA>
int launch_typed_w(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s)
{
    static int bps = 0;
    if (!bps) {
        int b = 0;
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, mpw_frame_kernel<G, Q, FRACTAL, JULIA>, kMpwBlock, 0));
        bps = b < 1 ? 1 : b;
    }
    const long pixels = p.list ? (long)p.W * p.nrows : (long)p.W * p.nrows;
    long grid = (long)ctx->num_sms * bps;
    const long needed = (pixels + kMpwBlock / G - 1) / (kMpwBlock / G);
    if (grid > needed)
        grid = needed;
    if (grid < 1)
        grid = 1;
    mpw_frame_kernel<G, Q, FRACTAL, JULIA><<<(unsigned)grid, kMpwBlock, 0, s>>>(p);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

template <int G, int Q>
int preload_w()
{
    int b = 0;
    MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &b, mpw_frame_kernel<G, Q, MDZ_MANDELBROT, false>, kMpwBlock, 0));
    MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &b, mpw_frame_kernel<G, Q, MDZ_BURNING_SHIP, false>, kMpwBlock, 0));
    MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &b, mpw_frame_kernel<G, Q, MDZ_GENERALIZED_CELTIC, false>, kMpwBlock, 0));
    MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &b, mpw_frame_kernel<G, Q, MDZ_VARIANT, false>, kMpwBlock, 0));
    return MDZGPU_OK;
}

}  // namespace

template <int G, int Q>
int launch_wide(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s)
{
    const bool julia = p.family == MDZ_FAMILY_JULIA;
    switch (p.fractal) {
    case MDZ_BURNING_SHIP:
        return julia ? launch_typed_w<G, Q, MDZ_BURNING_SHIP, true>(ctx, p, s)
                     : launch_typed_w<G, Q, MDZ_BURNING_SHIP, false>(ctx, p, s);
    case MDZ_GENERALIZED_CELTIC:
        return julia ? launch_typed_w<G, Q, MDZ_GENERALIZED_CELTIC, true>(ctx, p, s)
                     : launch_typed_w<G, Q, MDZ_GENERALIZED_CELTIC, false>(ctx, p, s);
    case MDZ_VARIANT:
        return julia ? launch_typed_w<G, Q, MDZ_VARIANT, true>(ctx, p, s)
                     : launch_typed_w<G, Q, MDZ_VARIANT, false>(ctx, p, s);
    default:
        return julia ? launch_typed_w<G, Q, MDZ_MANDELBROT, true>(ctx, p, s)
                     : launch_typed_w<G, Q, MDZ_MANDELBROT, false>(ctx, p, s);
    }
}

template <int G, int Q>
int preload_wide()
{
    return preload_w<G, Q>();
}

#if defined(MDZ_MPW_G) && defined(MDZ_MPW_Q)
template int launch_wide<MDZ_MPW_G, MDZ_MPW_Q>(mdzgpu_ctx*, const MpLaunch&, cudaStream_t);
template int preload_wide<MDZ_MPW_G, MDZ_MPW_Q>();
#endif

}  // namespace mdz

