// Multi-limb fixed-point escape-time kernel: the GPU form of MDZ's
// multiprecision path.
//
// Reference loops (per iteration, same operation order):
//   Mandelbrot          src/frac_mandel.c:25-52        (MPFR)  :55-82  (GMP)
//   burning ship        src/frac_burning_ship.c:27-55  (MPFR)  :58-86  (GMP)
//   generalized celtic  src/frac_generalized_celtic.c:27-55    :58-86
//   hybrid              src/frac_variant.c:26-55               :58-87
//   pixel -> coordinate src/fractal.c:159-192 (MPFR), :299-332 (GMP)
// MPFR/GMP floats are replaced by N-word fixed point (fixed_point.cuh) with
// at least precision+8 bits; counts agree with MPFR at the same precision
// wherever MPFR at twice the precision agrees with it.
//
// One thread iterates one pixel; magnitudes and sign masks are kept
// separately so the three products per iteration run on magnitudes.  c stays
// in registers up to 16 words and moves to shared memory above that so the
// 34/36-word (1088-bit class) kernels fit in registers.  Work is pulled in
// 8x4 tiles per warp from an atomic counter, as in the FP64 kernel.
#include "fixed_point.cuh"
#include "internal.h"
#include "serve.h"

namespace mdz {
namespace {

constexpr int kTileW = 8;
constexpr int kTileH = 4;

template <int N>
struct CRegs {
    uint32_t w[N];
    __device__ __forceinline__ uint32_t operator()(int k) const { return w[k]; }
};

template <int N>
struct CShared {
    const uint32_t* base;  // word k of this thread at base[k * stride]
    int stride;
    __device__ __forceinline__ uint32_t operator()(int k) const { return base[k * stride]; }
};

// Top two words of a fixed-point number as a float (value < 128 in size).
template <int N>
__device__ __forceinline__ float fx_top_float(const uint32_t (&x)[N])
{
    return (float)(int32_t)x[N - 1] * 5.9604645e-8f /* 2^-24 */
           + (float)x[N - 2] * 1.3877788e-17f /* 2^-56 */;
}

template <int N, int FRACTAL, class CG>
__device__ __forceinline__ uint32_t escape_mp(uint32_t (&wre)[N], uint32_t (&wim)[N],
                                              const CG& c_re, const CG& c_im, uint32_t depth,
                                              float& mag)
{
    uint32_t wre2[N], wim2[N], acc[N + 2], t[N], d[N];
    uint32_t sre = fx::abs_inplace<N>(wre);
    uint32_t sim = fx::abs_inplace<N>(wim);
    fx::sqr_trunc<N>(wre, acc);
    fx::extract<N, 24>(acc, wre2);
    fx::sqr_trunc<N>(wim, acc);
    fx::extract<N, 24>(acc, wim2);
    for (uint32_t wz = 1; wz <= depth; ++wz) {
        // wim = 2.0 * wre * wim + c_im   (burning ship: 2 |wre wim| + c_im)
        fx::mul_trunc<N>(wre, wim, acc);
        fx::extract<N, 23>(acc, t);
        const uint32_t mt = (FRACTAL == MDZ_BURNING_SHIP) ? 0u : (sre ^ sim);
        fx::add_signed<N>(c_im, t, mt, wim);
        // wre = wre2 - wim2 + c_re       (celtic: |wre2 - wim2| + c_re)
        fx::sub<N>(wre2, wim2, d);
        uint32_t md = 0u;
        if (FRACTAL == MDZ_GENERALIZED_CELTIC || (FRACTAL == MDZ_VARIANT && (wz & 1u)))
            md = (uint32_t)((int32_t)d[N - 1] >> 31);
        fx::add_signed<N>(c_re, d, md, wre);
        if (fx::big<N>(wre) || fx::big<N>(wim)) {
            const float a = fx_top_float<N>(wre), b = fx_top_float<N>(wim);
            mag = a * a + b * b;
            return wz;
        }
        sre = fx::abs_inplace<N>(wre);
        sim = fx::abs_inplace<N>(wim);
        // wim2 = wim * wim; wre2 = wre * wre
        fx::sqr_trunc<N>(wim, acc);
        fx::extract<N, 24>(acc, wim2);
        fx::sqr_trunc<N>(wre, acc);
        fx::extract<N, 24>(acc, wre2);
        if (fx::sum_gt4<N>(wim2, wre2)) {
            mag = fx_top_float<N>(wim2) + fx_top_float<N>(wre2);
            return wz;
        }
    }
    mag = fx_top_float<N>(wim2) + fx_top_float<N>(wre2);
    return 0;
}

// Resumable form for the serving engine: enters with |wre|, |wim| and their
// sign masks after iteration wz - 1, runs iterations wz .. last (<= depth)
// with the formula chosen at run time, and returns true when the pixel is
// finished (count in wz: the escape iteration, or 0 at depth); false leaves
// the state after iteration `last` (wz = last + 1).  The operations are
// those of escape_mp, so a pixel split over any number of calls gets the
// same count.
template <int N, class CG>
__device__ __forceinline__ bool escape_mp_resume(uint32_t (&wre)[N], uint32_t (&wim)[N],
                                                 uint32_t& sre, uint32_t& sim, const CG& c_re,
                                                 const CG& c_im, int fractal, uint32_t& wz,
                                                 uint32_t last, uint32_t depth, float& mag)
{
    uint32_t wre2[N], wim2[N], acc[N + 2], t[N], d[N];
    fx::sqr_trunc<N>(wre, acc);
    fx::extract<N, 24>(acc, wre2);
    fx::sqr_trunc<N>(wim, acc);
    fx::extract<N, 24>(acc, wim2);
    const bool ship = fractal == MDZ_BURNING_SHIP;
    const bool celtic = fractal == MDZ_GENERALIZED_CELTIC;
    const bool variant = fractal == MDZ_VARIANT;
    if (last > depth)
        last = depth;
    for (; wz <= last; ++wz) {
        fx::mul_trunc<N>(wre, wim, acc);
        fx::extract<N, 23>(acc, t);
        const uint32_t mt = ship ? 0u : (sre ^ sim);
        fx::add_signed<N>(c_im, t, mt, wim);
        fx::sub<N>(wre2, wim2, d);
        uint32_t md = 0u;
        if (celtic || (variant && (wz & 1u)))
            md = (uint32_t)((int32_t)d[N - 1] >> 31);
        fx::add_signed<N>(c_re, d, md, wre);
        if (fx::big<N>(wre) || fx::big<N>(wim)) {
            const float a = fx_top_float<N>(wre), b = fx_top_float<N>(wim);
            mag = a * a + b * b;
            return true;
        }
        sre = fx::abs_inplace<N>(wre);
        sim = fx::abs_inplace<N>(wim);
        fx::sqr_trunc<N>(wim, acc);
        fx::extract<N, 24>(acc, wim2);
        fx::sqr_trunc<N>(wre, acc);
        fx::extract<N, 24>(acc, wre2);
        if (fx::sum_gt4<N>(wim2, wre2)) {
            mag = fx_top_float<N>(wim2) + fx_top_float<N>(wre2);
            return true;
        }
    }
    mag = fx_top_float<N>(wim2) + fx_top_float<N>(wre2);
    if (wz > depth) {
        wz = 0;
        return true;
    }
    return false;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int N>
__host__ __device__ constexpr bool c_in_smem()
{
    return N > 16;
}

template <int N>
__host__ __device__ constexpr int block_threads()
{
    return N > 16 ? 128 : 256;
}

template <int N, int FRACTAL, bool JULIA>
__global__ void __launch_bounds__(block_threads<N>()) mp_frame_kernel(MpLaunch p)
{
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31;
    const int tiles_x = (p.W + kTileW - 1) / kTileW;
    const int tiles_y = (p.nrows + kTileH - 1) / kTileH;
    const unsigned list_n = p.list ? *p.list_count : 0u;
    const unsigned total = p.list ? (list_n + 31u) / 32u : (unsigned)tiles_x * (unsigned)tiles_y;
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
        int ix, lrow, ty = 0;
        bool valid;
        if (p.list) {
            const unsigned i = tile * 32u + lane;
            valid = i < list_n;
            const unsigned pix = valid ? p.list[i] : 0u;
            lrow = (int)(pix / (unsigned)p.W);
            ix = (int)(pix - (unsigned)lrow * (unsigned)p.W);
        } else {
            ty = (int)(tile / (unsigned)tiles_x);
            const int tx = (int)(tile - (unsigned)ty * (unsigned)tiles_x);
            ix = tx * kTileW + (lane & (kTileW - 1));
            lrow = ty * kTileH + (lane / kTileW);
            valid = ix < p.W && lrow < p.nrows;
        }
        unsigned long long its = 0;
        if (valid) {
            uint32_t wre[N], wim[N];
            const uint32_t* xs = p.xs + (size_t)ix * N;
            const uint32_t* ys = p.ys + (size_t)lrow * N;
#pragma unroll
            for (int k = 0; k < N; ++k) {
                wre[k] = xs[k];
                wim[k] = ys[k];
            }
            uint32_t n;
            float mag = 0.f;
            if constexpr (c_in_smem<N>()) {
                const int stride = blockDim.x;
                uint32_t* cre = smem + threadIdx.x;
                uint32_t* cim = smem + (size_t)N * stride + threadIdx.x;
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    cre[k * stride] = JULIA ? p.julia[k] : wre[k];
                    cim[k * stride] = JULIA ? p.julia[N + k] : wim[k];
                }
                CShared<N> gr{cre, stride}, gi{cim, stride};
                n = escape_mp<N, FRACTAL>(wre, wim, gr, gi, p.depth, mag);
            } else {
                CRegs<N> gr, gi;
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    gr.w[k] = JULIA ? p.julia[k] : wre[k];
                    gi.w[k] = JULIA ? p.julia[N + k] : wim[k];
                }
                n = escape_mp<N, FRACTAL>(wre, wim, gr, gi, p.depth, mag);
            }
            p.out[(size_t)lrow * p.W + ix] = (int32_t)n;
            if (p.mag)
                p.mag[(size_t)lrow * p.W + ix] = mag;
            its = n ? n : p.depth;
        }
        its = warp_sum_u64(its);
        if (p.band_flags)
            __threadfence_system();
        __syncwarp();
        if (lane == 0) {
            atomicAdd(&p.sync->iter_sum, its);
            if (p.tile_rows_done && !p.list) {
                const unsigned done = atomicAdd(&p.tile_rows_done[ty], 1u) + 1u;
                if (done == (unsigned)tiles_x && p.band_flags) {
                    __threadfence_system();
                    p.band_flags[ty] = 1;
                }
            }
        }
    }
    if (p.done.count)
        done_signal(p.done, (unsigned long long)p.tile_base + p.tile_limit >= total ? 3 : 1);
}

// Serving: one step of the multi-limb method over its mixed work queue
// (class `cls`); see serve.h.  State per pixel: |wre| (N words), |wim| (N
// words), the next iteration, the two sign masks.
template <int N>
__global__ void __launch_bounds__(block_threads<N>()) serve_mp_kernel(ServeDev* __restrict__ d,
                                                                     int cls)
{
    extern __shared__ uint32_t smem[];
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
                const int W = rq.pl.W;
                const int line = (int)(pix / (unsigned)W);
                const int ix = (int)(pix - (unsigned)line * (unsigned)W);
                const uint32_t* xs = rq.xs + (size_t)ix * N;
                const uint32_t* ys = rq.ys + (size_t)line * N;
                // c: the pixel (Mandelbrot family) or the Julia constant
                const uint32_t* cxs = rq.julia ? rq.julia : xs;
                const uint32_t* cys = rq.julia ? rq.julia + N : ys;
                uint32_t* sp = (uint32_t*)(rq.state + (size_t)pix * rq.state_stride);
                uint32_t wre[N], wim[N], sre, sim, wz;
                if (e & kEntryFresh) {
#pragma unroll
                    for (int k = 0; k < N; ++k) {
                        wre[k] = xs[k];
                        wim[k] = ys[k];
                    }
                    sre = fx::abs_inplace<N>(wre);
                    sim = fx::abs_inplace<N>(wim);
                    wz = 1;
                } else {
#pragma unroll
                    for (int k = 0; k < N; ++k) {
                        wre[k] = sp[k];
                        wim[k] = sp[N + k];
                    }
                    wz = sp[2 * N];
                    const uint32_t sg = sp[2 * N + 1];
                    sre = (sg & 1u) ? 0xffffffffu : 0u;
                    sim = (sg & 2u) ? 0xffffffffu : 0u;
                }
                const uint32_t last = wz + d->ctl.budget[slot] - 1u;
                const uint32_t depth = rq.pl.depth;
                float mag = 0.f;
                bool fin;
                if constexpr (c_in_smem<N>()) {
                    const int stride = blockDim.x;
                    uint32_t* cre = smem + threadIdx.x;
                    uint32_t* cim = smem + (size_t)N * stride + threadIdx.x;
#pragma unroll
                    for (int k = 0; k < N; ++k) {
                        cre[k * stride] = cxs[k];
                        cim[k * stride] = cys[k];
                    }
                    CShared<N> gr{cre, stride}, gi{cim, stride};
                    fin = escape_mp_resume<N>(wre, wim, sre, sim, gr, gi, rq.fractal, wz, last,
                                              depth, mag);
                } else {
                    CRegs<N> gr, gi;
#pragma unroll
                    for (int k = 0; k < N; ++k) {
                        gr.w[k] = cxs[k];
                        gi.w[k] = cys[k];
                    }
                    fin = escape_mp_resume<N>(wre, wim, sre, sim, gr, gi, rq.fractal, wz, last,
                                              depth, mag);
                }
                if (fin) {
                    rq.pl.out[pix] = (int32_t)wz;
                    if (rq.pl.mag)
                        rq.pl.mag[pix] = mag;
                    done = true;
                } else {
#pragma unroll
                    for (int k = 0; k < N; ++k) {
                        sp[k] = wre[k];
                        sp[N + k] = wim[k];
                    }
                    sp[2 * N] = wz;
                    sp[2 * N + 1] = (sre & 1u) | (sim & 2u);
                    again = true;
                }
            }
        }
        // warp-aggregated append of the unfinished pixels
        const unsigned amask = __ballot_sync(0xffffffffu, again);
        if (amask) {
            const int leader = __ffs(amask) - 1;
            unsigned b = 0;
            if (lane == leader)
                b = atomicAdd(qout_count, (unsigned)__popc(amask));
            b = __shfl_sync(0xffffffffu, b, leader);
            if (again)
                qout[b + __popc(amask & ((1u << lane) - 1u))] = e & ~kEntryFresh;
        }
        const unsigned dmask = __ballot_sync(0xffffffffu, done);
        if (done) {
            const unsigned grp = __match_any_sync(dmask, slot);
            if (lane == __ffs(grp) - 1)
                atomicSub(d->status.remaining + slot, (unsigned)__popc(grp));
        }
    }
}

// Attributes and occupancy of one frame kernel, set up once.  The first
// call also loads the kernel (with lazy module loading, a load waits for
// the work running on the device, so servers call it before they start).
template <int N, int FRACTAL, bool JULIA>
int typed_blocks_per_sm(int* out)
{
    constexpr int threads = block_threads<N>();
    const size_t smem = c_in_smem<N>() ? (size_t)2 * N * threads * sizeof(uint32_t) : 0;
    static int blocks_per_sm = 0;
    if (!blocks_per_sm) {
        if (smem > 48 * 1024)
            MDZ_CUDA_TRY(cudaFuncSetAttribute(mp_frame_kernel<N, FRACTAL, JULIA>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
        int b = 0;
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, mp_frame_kernel<N, FRACTAL, JULIA>, threads, smem));
        blocks_per_sm = b < 1 ? 1 : b;
    }
    *out = blocks_per_sm;
    return MDZGPU_OK;
}

template <int N, int FRACTAL, bool JULIA>
int launch_typed(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s)
{
    constexpr int threads = block_threads<N>();
    const size_t smem = c_in_smem<N>() ? (size_t)2 * N * threads * sizeof(uint32_t) : 0;
    int blocks_per_sm = 1;
    if (int rc = typed_blocks_per_sm<N, FRACTAL, JULIA>(&blocks_per_sm))
        return rc;
    const long tiles = p.list ? ((long)p.W * p.nrows + 31) / 32
                              : (long)((p.W + kTileW - 1) / kTileW) * ((p.nrows + kTileH - 1) / kTileH);
    long grid = (long)ctx->num_sms * blocks_per_sm;
    const long blocks_needed = (tiles + threads / 32 - 1) / (threads / 32);
    if (grid > blocks_needed)
        grid = blocks_needed;
    if (grid < 1)
        grid = 1;
    mp_frame_kernel<N, FRACTAL, JULIA><<<(unsigned)grid, threads, smem, s>>>(p);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

}  // namespace

template <int N>
int launch_words(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s)
{
    const bool julia = p.family == MDZ_FAMILY_JULIA;
    switch (p.fractal) {
    case MDZ_BURNING_SHIP:
        return julia ? launch_typed<N, MDZ_BURNING_SHIP, true>(ctx, p, s)
                     : launch_typed<N, MDZ_BURNING_SHIP, false>(ctx, p, s);
    case MDZ_GENERALIZED_CELTIC:
        return julia ? launch_typed<N, MDZ_GENERALIZED_CELTIC, true>(ctx, p, s)
                     : launch_typed<N, MDZ_GENERALIZED_CELTIC, false>(ctx, p, s);
    case MDZ_VARIANT:
        return julia ? launch_typed<N, MDZ_VARIANT, true>(ctx, p, s)
                     : launch_typed<N, MDZ_VARIANT, false>(ctx, p, s);
    default:
        return julia ? launch_typed<N, MDZ_MANDELBROT, true>(ctx, p, s)
                     : launch_typed<N, MDZ_MANDELBROT, false>(ctx, p, s);
    }
}


template <int N>
int launch_serve_mp_words(ServeDev* d, int mp_class, int num_sms, cudaStream_t s)
{
    constexpr int threads = block_threads<N>();
    const size_t smem = c_in_smem<N>() ? (size_t)2 * N * threads * sizeof(uint32_t) : 0;
    static int bps = 0;
    if (!bps) {
        if (smem > 48 * 1024)
            MDZ_CUDA_TRY(cudaFuncSetAttribute(serve_mp_kernel<N>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, serve_mp_kernel<N>,
                                                                   threads, smem));
        if (bps < 1)
            bps = 1;
    }
    serve_mp_kernel<N><<<(unsigned)(num_sms * bps), threads, smem, s>>>(d, mp_class);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

template <int N>
int preload_words()
{
    int b = 0, rc = MDZGPU_OK;
    for (int j = 0; j < 2 && !rc; ++j) {
        const bool julia = j == 1;
        rc = julia ? typed_blocks_per_sm<N, MDZ_MANDELBROT, true>(&b)
                   : typed_blocks_per_sm<N, MDZ_MANDELBROT, false>(&b);
        if (!rc)
            rc = julia ? typed_blocks_per_sm<N, MDZ_BURNING_SHIP, true>(&b)
                       : typed_blocks_per_sm<N, MDZ_BURNING_SHIP, false>(&b);
        if (!rc)
            rc = julia ? typed_blocks_per_sm<N, MDZ_GENERALIZED_CELTIC, true>(&b)
                       : typed_blocks_per_sm<N, MDZ_GENERALIZED_CELTIC, false>(&b);
        if (!rc)
            rc = julia ? typed_blocks_per_sm<N, MDZ_VARIANT, true>(&b)
                       : typed_blocks_per_sm<N, MDZ_VARIANT, false>(&b);
    }
    return rc;
}

#ifdef MDZ_MP_WORDS
// One translation unit per word count (the build compiles this file once for
// every count in the list) keeps the large unrolled kernels compiling in
// parallel.
template int launch_words<MDZ_MP_WORDS>(mdzgpu_ctx*, const MpLaunch&, cudaStream_t);
template int launch_serve_mp_words<MDZ_MP_WORDS>(ServeDev*, int, int, cudaStream_t);
template int preload_words<MDZ_MP_WORDS>();
#endif

}  // namespace mdz
