// FP64 escape-time kernel: the GPU form of MDZ's hardware-float path.
//
// Arithmetic follows, operation for operation, the reference built with
// `long double` = IEEE double and no FMA contraction:
//   pixel -> coordinate  src/fractal.c:50-77
//   Mandelbrot           src/frac_mandel.c:5-21
//   burning ship         src/frac_burning_ship.c:7-24
//   generalized celtic   src/frac_generalized_celtic.c:7-24
//   mandel-celtic hybrid src/frac_variant.c:5-24
// Every operation is an explicit __dmul_rn / __dadd_rn / __dsub_rn /
// __ddiv_rn, which the compiler never fuses, so the counts are bit-exact
// whatever -fmad says.
//
// Work split (the GPU form of src/render_threads.c:360-393): instead of a
// mutex-protected next_line counter advanced by whole rows, each warp pulls
// an 8x4 pixel tile from a global atomic counter.  Square-ish tiles keep the
// 32 lanes of a warp on neighbouring pixels, whose counts are close, which
// limits divergence; dynamic pulling balances the very uneven rows.  When a
// 4-row band completes, the warp that finished it raises a host-visible
// band flag (the analogue of lines_rendered[] + lines_rendered_cond).
#include "internal.h"

namespace mdz {
namespace {

constexpr int kTileW = 8;
constexpr int kTileH = 4;
constexpr int kBlock = 256;

template <int FRACTAL, bool JULIA>
__device__ __forceinline__ uint32_t escape_fp64(double x, double y, double jre,
                                                double jim, uint32_t depth)
{
    double wre = x, wim = y;
    double wre2 = __dmul_rn(x, x);
    double wim2 = __dmul_rn(y, y);
    const double c_re = JULIA ? jre : x;
    const double c_im = JULIA ? jim : y;
    for (uint32_t wz = 1; wz <= depth; ++wz) {
        double t;
        if (FRACTAL == MDZ_BURNING_SHIP)
            t = __dmul_rn(2.0, fabs(__dmul_rn(wre, wim)));  // 2.0 * fabsl(wre * wim)
        else
            t = __dmul_rn(__dmul_rn(2.0, wre), wim);         // 2.0 * wre * wim
        wim = __dadd_rn(t, c_im);
        double d = __dsub_rn(wre2, wim2);
        if (FRACTAL == MDZ_GENERALIZED_CELTIC || (FRACTAL == MDZ_VARIANT && (wz & 1u)))
            d = fabs(d);
        wre = __dadd_rn(d, c_re);
        wim2 = __dmul_rn(wim, wim);
        wre2 = __dmul_rn(wre, wre);
        if (__dadd_rn(wim2, wre2) > 4.0)
            return wz;
    }
    return 0;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int FRACTAL, bool JULIA>
__global__ void __launch_bounds__(kBlock) fp64_frame_kernel(Fp64Launch p)
{
    const int lane = threadIdx.x & 31;
    const int tiles_x = (p.W + kTileW - 1) / kTileW;
    const int tiles_y = (p.nrows + kTileH - 1) / kTileH;
    const unsigned total = (unsigned)tiles_x * (unsigned)tiles_y;
    const double width = __dsub_rn(p.xmax, p.xmin);
    const double fw = (double)p.W;
    const double ystep = __ddiv_rn(width, fw);
    for (;;) {
        unsigned t = 0;
        if (lane == 0)
            t = (p.stop && *p.stop) ? total : atomicAdd(&p.sync->tile_counter, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total)
            break;
        const int ty = (int)(t / (unsigned)tiles_x);
        const int tx = (int)(t - (unsigned)ty * (unsigned)tiles_x);
        const int ix = tx * kTileW + (lane & (kTileW - 1));
        const int lrow = ty * kTileH + (lane / kTileW);
        unsigned long long its = 0;
        if (ix < p.W && lrow < p.nrows) {
            const int line = p.row0 + lrow;
            const double y = __dsub_rn(p.ymax, __dmul_rn(ystep, (double)line));
            const double x =
                __dadd_rn(__dmul_rn(__ddiv_rn((double)ix, fw), width), p.xmin);
            const uint32_t n = escape_fp64<FRACTAL, JULIA>(x, y, p.jre, p.jim, p.depth);
            p.out[(size_t)lrow * p.W + ix] = (int32_t)n;
            its = n ? n : p.depth;
        }
        its = warp_sum_u64(its);
        if (p.band_flags)
            __threadfence_system();
        __syncwarp();
        if (lane == 0) {
            atomicAdd(&p.sync->iter_sum, its);
            if (p.tile_rows_done) {
                const unsigned done = atomicAdd(&p.tile_rows_done[ty], 1u) + 1u;
                if (done == (unsigned)tiles_x && p.band_flags) {
                    __threadfence_system();
                    p.band_flags[ty] = 1;
                }
            }
        }
    }
}

template <int FRACTAL, bool JULIA>
int launch_one(mdzgpu_ctx* ctx, const Fp64Launch& p, cudaStream_t s)
{
    static int blocks_per_sm = 0;
    if (!blocks_per_sm) {
        MDZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &blocks_per_sm, fp64_frame_kernel<FRACTAL, JULIA>, kBlock, 0));
        if (blocks_per_sm < 1)
            blocks_per_sm = 1;
    }
    const long tiles = (long)((p.W + kTileW - 1) / kTileW) * ((p.nrows + kTileH - 1) / kTileH);
    long grid = (long)ctx->num_sms * blocks_per_sm;
    const long warps_needed = tiles;
    const long blocks_needed = (warps_needed + kBlock / 32 - 1) / (kBlock / 32);
    if (grid > blocks_needed)
        grid = blocks_needed;
    if (grid < 1)
        grid = 1;
    fp64_frame_kernel<FRACTAL, JULIA><<<(unsigned)grid, kBlock, 0, s>>>(p);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

}  // namespace

int launch_fp64(mdzgpu_ctx* ctx, const Fp64Launch& p, cudaStream_t s)
{
    const bool julia = p.family == MDZ_FAMILY_JULIA;
    switch (p.fractal) {
    case MDZ_BURNING_SHIP:
        return julia ? launch_one<MDZ_BURNING_SHIP, true>(ctx, p, s)
                     : launch_one<MDZ_BURNING_SHIP, false>(ctx, p, s);
    case MDZ_GENERALIZED_CELTIC:
        return julia ? launch_one<MDZ_GENERALIZED_CELTIC, true>(ctx, p, s)
                     : launch_one<MDZ_GENERALIZED_CELTIC, false>(ctx, p, s);
    case MDZ_VARIANT:
        return julia ? launch_one<MDZ_VARIANT, true>(ctx, p, s)
                     : launch_one<MDZ_VARIANT, false>(ctx, p, s);
    default:  // MANDELBROT and anything else, as the reference's `default:`
        return julia ? launch_one<MDZ_MANDELBROT, true>(ctx, p, s)
                     : launch_one<MDZ_MANDELBROT, false>(ctx, p, s);
    }
}

}  // namespace mdz
