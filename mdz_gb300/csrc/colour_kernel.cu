// Colouring epilogue: MDZ's palette_apply (src/palette.c:406-463) for
// aa = 1 and do_anti_aliasing (src/render.c:108-158) through
// get_pixel_colour (src/palette.c:466-503) for aa > 1, on the GPU, so that
// only the RGB image (user_w x user_h x 4 bytes) leaves the device.
//
// One thread per output pixel; the palette (<= 256 colours) is staged in
// shared memory.  Every double is formed as the reference's C code forms it
// (explicit _rn operations, no contraction), every conversion truncates as
// C's casts do, so the colours are identical to the reference's on the
// domain 0 <= count * colour_scale + offset < 2^31.
#include "internal.h"

namespace mdz {
namespace {

__device__ __forceinline__ uint32_t red(uint32_t x) { return x & 0xffu; }
__device__ __forceinline__ uint32_t green(uint32_t x) { return (x & 0xff00u) >> 8; }
__device__ __forceinline__ uint32_t blue(uint32_t x) { return (x & 0xff0000u) >> 16; }
__device__ __forceinline__ uint32_t pack(uint32_t r, uint32_t g, uint32_t b)
{
    return r | (g << 8) | (b << 16);
}

// (guint32) of a double in [0, 2^31)
__device__ __forceinline__ uint32_t to_u32(double v)
{
    return (uint32_t)__double2ll_rz(v);
}

// (guint8) of a blend in [0, 256)
__device__ __forceinline__ uint32_t to_u8(double v)
{
    return (uint32_t)__double2int_rz(v) & 0xffu;
}

// diff * X(c1) + rdiff * X(c2), the reference's interpolation, per channel
__device__ __forceinline__ uint32_t blend(double diff, double rdiff, uint32_t c1, uint32_t c2)
{
    const uint32_t r = to_u8(__dadd_rn(__dmul_rn(diff, (double)red(c1)),
                                       __dmul_rn(rdiff, (double)red(c2))));
    const uint32_t g = to_u8(__dadd_rn(__dmul_rn(diff, (double)green(c1)),
                                       __dmul_rn(rdiff, (double)green(c2))));
    const uint32_t b = to_u8(__dadd_rn(__dmul_rn(diff, (double)blue(c1)),
                                       __dmul_rn(rdiff, (double)blue(c2))));
    return pack(r, g, b);
}

// get_pixel_colour(raw * scale, ip)
__device__ __forceinline__ uint32_t pixel_colour(double val, int ip, const uint32_t* pal,
                                                 uint32_t m, int off)
{
    if (val != 0.0)
        val = __dadd_rn(val, (double)off);
    if (ip) {
        const double cval = ceil(val);
        const double diff = __dsub_rn(cval, val);
        const double rdiff = __dsub_rn(1.0, diff);
        const uint32_t i1 = to_u32(floor(val)) % m;
        const uint32_t i2 = to_u32(cval) % m;
        return blend(diff, rdiff, pal[i1], pal[i2]);
    }
    if (val == 0.0)
        return 0u;
    return pal[to_u32(val) % m];
}

__global__ void __launch_bounds__(256) colour_kernel(const int32_t* __restrict__ raw, int real_w,
                                                     int user_w, int user_h, int aa, int ip,
                                                     double scale, const uint32_t* palette,
                                                     int n, int off, uint32_t* __restrict__ rgb)
{
    __shared__ uint32_t pal[256];
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        pal[i] = palette[i];
    __syncthreads();
    const uint32_t m = (uint32_t)(n - 1);
    const long total = (long)user_w * user_h;
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < total;
         p += (long)gridDim.x * blockDim.x) {
        const int y = (int)(p / user_w), x = (int)(p - (long)y * user_w);
        uint32_t out = 0;
        if (aa == 1) {
            // palette_apply
            const int v = raw[(size_t)y * real_w + x];
            if (v) {
                const double ip_val = __dadd_rn(__dmul_rn((double)v, scale), (double)off);
                if (ip) {
                    const int ip_cval = __double2int_rz(ceil(ip_val));
                    const double ip_diff = __dsub_rn((double)ip_cval, ip_val);
                    const double ip_rdiff = __dsub_rn(1.0, ip_diff);
                    const int i1 = __double2int_rz(floor(ip_val)) % (n - 1);
                    const int i2 = ip_cval % (n - 1);
                    out = blend(ip_diff, ip_rdiff, pal[i1], pal[i2]);
                } else {
                    out = pal[to_u32(ip_val) % m];
                }
            }
        } else {
            // do_anti_aliasing: channel sums over the aa x aa block, then
            // integer division
            uint32_t r = 0, g = 0, b = 0;
            for (int yi = y * aa; yi < y * aa + aa; ++yi) {
                const int32_t* row = raw + (size_t)yi * real_w;
                for (int xi = x * aa; xi < x * aa + aa; ++xi) {
                    const uint32_t c =
                        pixel_colour(__dmul_rn((double)row[xi], scale), ip, pal, m, off);
                    r += red(c);
                    g += green(c);
                    b += blue(c);
                }
            }
            const uint32_t a2 = (uint32_t)(aa * aa);
            out = pack(r / a2, g / a2, b / a2);
        }
        rgb[p] = out;
    }
}

int check_palette(const mdzgpu_palette* pal, int real_w, int real_h, int aa)
{
    if (!pal || !pal->colours || pal->indexes < 2 || pal->indexes > 256) {
        set_error("colour: palette needs 2..256 colours");
        return MDZGPU_ERR_ARG;
    }
    if (aa < 1 || real_w <= 0 || real_h <= 0 || real_w % aa || real_h % aa) {
        set_error("colour: %d x %d counts are not whole %d x %d blocks", real_w, real_h, aa, aa);
        return MDZGPU_ERR_ARG;
    }
    return MDZGPU_OK;
}

}  // namespace

int launch_colour(mdzgpu_ctx* ctx, const int32_t* d_raw, int real_w, int real_h, int aa,
                  const mdzgpu_palette* pal, const uint32_t* d_palette, uint32_t* d_rgb,
                  cudaStream_t s)
{
    const int uw = real_w / aa, uh = real_h / aa;
    const long total = (long)uw * uh;
    long blocks = (total + 255) / 256;
    const long cap = (long)ctx->num_sms * 8;
    if (blocks > cap)
        blocks = cap;
    if (blocks < 1)
        blocks = 1;
    colour_kernel<<<(unsigned)blocks, 256, 0, s>>>(d_raw, real_w, uw, uh, aa, pal->interpolate,
                                                   pal->colour_scale, d_palette, pal->indexes,
                                                   pal->offset, d_rgb);
    MDZ_CUDA_TRY(cudaGetLastError());
    return MDZGPU_OK;
}

}  // namespace mdz

using namespace mdz;

extern "C" int mdzgpu_colour_device(mdzgpu_ctx* ctx, const int32_t* d_counts, int32_t real_w,
                                    int32_t real_h, int32_t aa, const mdzgpu_palette* pal,
                                    uint32_t* d_rgb)
{
    if (!ctx || !d_counts || !d_rgb) {
        set_error("colour: null argument");
        return MDZGPU_ERR_ARG;
    }
    int rc = check_palette(pal, real_w, real_h, aa);
    if (rc)
        return rc;
    MDZ_CUDA_TRY(cudaSetDevice(ctx->device));
    if ((rc = ctx->palette.ensure(256 * sizeof(uint32_t))))
        return rc;
    MDZ_CUDA_TRY(cudaMemcpyAsync(ctx->palette.ptr, pal->colours, pal->indexes * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, ctx->stream));
    rc = launch_colour(ctx, d_counts, real_w, real_h, aa, pal, (const uint32_t*)ctx->palette.ptr,
                       d_rgb, ctx->stream);
    if (rc)
        return rc;
    MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return MDZGPU_OK;
}

extern "C" int mdzgpu_colour(mdzgpu_ctx* ctx, const int32_t* counts, int32_t real_w,
                             int32_t real_h, int32_t aa, const mdzgpu_palette* pal,
                             uint32_t* rgb)
{
    if (!ctx || !counts || !rgb) {
        set_error("colour: null argument");
        return MDZGPU_ERR_ARG;
    }
    int rc = check_palette(pal, real_w, real_h, aa);
    if (rc)
        return rc;
    MDZ_CUDA_TRY(cudaSetDevice(ctx->device));
    const size_t n_in = (size_t)real_w * real_h, n_out = n_in / ((size_t)aa * aa);
    if ((rc = ctx->counts.ensure(n_in * 4)) || (rc = ctx->aux.ensure(n_out * 4))
        || (rc = ctx->palette.ensure(256 * sizeof(uint32_t))))
        return rc;
    MDZ_CUDA_TRY(cudaMemcpyAsync(ctx->counts.ptr, counts, n_in * 4, cudaMemcpyHostToDevice,
                                 ctx->stream));
    MDZ_CUDA_TRY(cudaMemcpyAsync(ctx->palette.ptr, pal->colours, pal->indexes * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, ctx->stream));
    rc = launch_colour(ctx, (const int32_t*)ctx->counts.ptr, real_w, real_h, aa, pal,
                       (const uint32_t*)ctx->palette.ptr, (uint32_t*)ctx->aux.ptr, ctx->stream);
    if (rc)
        return rc;
    MDZ_CUDA_TRY(cudaMemcpyAsync(rgb, ctx->aux.ptr, n_out * 4, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return MDZGPU_OK;
}
