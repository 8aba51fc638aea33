// Explicit-parameter C ABI of libmdzgpu (mdzgpu_*): contexts, frame renders
// for the FP64, multi-limb and perturbation methods.
#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <string>
#include <vector>

#include "internal.h"

namespace mdz {

namespace {
thread_local std::string g_last_error;

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

int validate_frame(const mdzgpu_frame* f)
{
    if (!f || f->width <= 0 || f->height <= 0 || f->width > 1 << 20 || f->height > 1 << 20) {
        set_error("invalid frame size");
        return MDZGPU_ERR_ARG;
    }
    if (f->depth < 1 || f->depth > 0x7fffffffLL) {
        set_error("depth %lld outside [1, INT32_MAX]", (long long)f->depth);
        return MDZGPU_ERR_ARG;
    }
    if (f->family != MDZ_FAMILY_MANDEL && f->family != MDZ_FAMILY_JULIA) {
        set_error("unknown family %d", f->family);
        return MDZGPU_ERR_ARG;
    }
    return MDZGPU_OK;
}

struct Timing {
    double t0;
    explicit Timing() : t0(now_ms()) {}
};

}  // namespace

void set_error(const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    fprintf(stderr, "mdzgpu: %s\n", buf);
}

int DevBuf::ensure(size_t want)
{
    if (want <= bytes && ptr)
        return MDZGPU_OK;
    release();
    size_t b = want < 256 ? 256 : want;
    cudaError_t e = cudaMalloc(&ptr, b);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        set_error("cudaMalloc(%zu): %s", b, cudaGetErrorString(e));
        return MDZGPU_ERR_NOMEM;
    }
    bytes = b;
    return MDZGPU_OK;
}

void DevBuf::release()
{
    if (ptr)
        cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

int PinnedBuf::ensure(size_t want)
{
    if (want <= bytes && host)
        return MDZGPU_OK;
    release();
    size_t b = want < 4096 ? 4096 : want;
    cudaError_t e = cudaHostAlloc(&host, b, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) {
        host = nullptr;
        set_error("cudaHostAlloc(%zu): %s", b, cudaGetErrorString(e));
        return MDZGPU_ERR_NOMEM;
    }
    e = cudaHostGetDevicePointer(&dev, host, 0);
    if (e != cudaSuccess) {
        cudaFreeHost(host);
        host = nullptr;
        set_error("cudaHostGetDevicePointer: %s", cudaGetErrorString(e));
        return MDZGPU_ERR_CUDA;
    }
    bytes = b;
    return MDZGPU_OK;
}

void PinnedBuf::release()
{
    if (host)
        cudaFreeHost(host);
    host = nullptr;
    dev = nullptr;
    bytes = 0;
}

int digits28_from_mpval(const mdzgpu_mpval* v, int L, int* out)
{
    // magnitude bits -> unsigned digits, then balance to [-2^27, 2^27)
    const long F = 28L * (L - 1);
    std::vector<long long> d(L + 1, 0);
    if (v && v->d && v->nlimbs > 0) {
        const long shift = (long)v->exp - 64L * v->nlimbs + F;
        for (int i = 0; i < v->nlimbs; ++i) {
            const uint64_t limb = v->d[i];
            for (int b = 0; b < 64; ++b) {
                if (!((limb >> b) & 1u))
                    continue;
                const long pos = (long)i * 64 + b + shift;
                if (pos < 0)
                    continue;
                if (pos >= 28L * L - 3)
                    return MDZGPU_ERR_RANGE;
                d[pos / 28] |= 1ll << (pos % 28);
            }
        }
    }
    if (v && v->sign < 0)
        for (auto& x : d)
            x = -x;
    for (int i = 0; i < L; ++i) {
        const long long digit = ((d[i] + (1ll << 27)) & ((1ll << 28) - 1)) - (1ll << 27);
        const long long carry = (d[i] - digit) >> 28;
        d[i] = digit;
        d[i + 1] += carry;
    }
    if (d[L] != 0)
        return MDZGPU_ERR_RANGE;
    for (int i = 0; i < L; ++i)
        out[i] = (int)d[i];
    return MDZGPU_OK;
}

int half_spacing(const mdzgpu_mpval* width, int W, double* hs_m, int* hs_e)
{
    if (!width || !width->d || width->nlimbs <= 0 || W <= 0) {
        set_error("perturbation needs a positive width");
        return MDZGPU_ERR_ARG;
    }
    // top 53 bits of the mantissa, as an integer-valued double
    const uint64_t top = width->d[width->nlimbs - 1];
    const double mant = (double)(top >> 11);            // exact, 53 bits
    const long e0 = (long)width->exp - 53;              // width ~ mant * 2^e0
    double q = mant / (2.0 * (double)W);
    const int k = ilogb(q);
    double m = ldexp(q, -k);                            // [1, 2)
    m = ldexp(nearbyint(ldexp(m, 39)), -39);            // 40 significant bits
    *hs_m = m;
    *hs_e = (int)(e0 + k);
    return MDZGPU_OK;
}

}  // namespace mdz

using namespace mdz;

extern "C" {

const char* mdzgpu_last_error(void)
{
    return g_last_error.c_str();
}

const char* mdzgpu_version(void)
{
    return "mdzgpu 0.1 (sm_103a)";
}

mdzgpu_ctx* mdzgpu_create(int device)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= device || device < 0) {
        set_error("no CUDA device %d (%s)", device, cudaGetErrorString(e));
        return nullptr;
    }
    if ((e = cudaSetDevice(device)) != cudaSuccess) {
        set_error("cudaSetDevice: %s", cudaGetErrorString(e));
        return nullptr;
    }
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) {
        set_error("cudaGetDeviceProperties: %s", cudaGetErrorString(e));
        return nullptr;
    }
    auto* ctx = new mdzgpu_ctx();
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess
        || cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, prio_hi) != cudaSuccess
        || cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess
        || cudaEventCreate(&ctx->ev_side0) != cudaSuccess
        || cudaEventCreate(&ctx->ev_k0) != cudaSuccess
        || cudaEventCreate(&ctx->ev_k1) != cudaSuccess) {
        set_error("stream/event creation failed");
        delete ctx;
        return nullptr;
    }
    return ctx;
}

void mdzgpu_destroy(mdzgpu_ctx* ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->counts.release();
    ctx->sync.release();
    ctx->coords.release();
    ctx->orbit.release();
    ctx->orbit_fx.release();
    ctx->aux.release();
    ctx->lists.release();
    ctx->pinned.release();
    ctx->staging.release();
    ctx->palette.release();
    ctx->pstate.release();
    ctx->pqueue.release();
    ctx->stepinfo.release();
    cudaStreamSynchronize(ctx->side);
    cudaEventDestroy(ctx->ev0);
    cudaEventDestroy(ctx->ev1);
    cudaEventDestroy(ctx->ev_side0);
    cudaEventDestroy(ctx->ev_k0);
    cudaEventDestroy(ctx->ev_k1);
    cudaStreamDestroy(ctx->side);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

static int finish_stats(mdzgpu_ctx* ctx, mdzgpu_stats* st, double t0, int launches,
                        int64_t h2d, int64_t d2h)
{
    FrameSync hs;
    MDZ_CUDA_TRY(cudaMemcpyAsync(&hs, ctx->sync.ptr, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream));
    MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (st) {
        float ms = 0.f;
        MDZ_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        st->kernel_ms = ms;
        st->pixel_iters = (int64_t)hs.iter_sum;
        st->launches = launches;
        st->h2d_bytes = h2d;
        st->d2h_bytes = d2h + (int64_t)sizeof hs;
        st->wall_ms = now_ms() - t0;
    }
    return MDZGPU_OK;
}

static int fp64_common(mdzgpu_ctx* ctx, const mdzgpu_frame* f, double xmin, double xmax,
                       double ymax, double jre, double jim, int32_t* d_out, int32_t* h_out,
                       mdzgpu_stats* st)
{
    const double t0 = now_ms();
    if (!ctx) {
        set_error("null context");
        return MDZGPU_ERR_ARG;
    }
    int rc = validate_frame(f);
    if (rc)
        return rc;
    MDZ_CUDA_TRY(cudaSetDevice(ctx->device));
    const size_t n = (size_t)f->width * f->height;
    if (!d_out) {
        if ((rc = ctx->counts.ensure(n * sizeof(int32_t))))
            return rc;
        d_out = (int32_t*)ctx->counts.ptr;
    }
    if ((rc = ctx->sync.ensure(sizeof(FrameSync))))
        return rc;
    if (st)
        memset(st, 0, sizeof *st);
    MDZ_CUDA_TRY(cudaMemsetAsync(ctx->sync.ptr, 0, sizeof(FrameSync), ctx->stream));
    Fp64Launch p;
    p.W = f->width;
    p.H = f->height;
    p.row0 = 0;
    p.nrows = f->height;
    p.family = f->family;
    p.fractal = f->fractal;
    p.depth = (uint32_t)f->depth;
    p.xmin = xmin;
    p.xmax = xmax;
    p.ymax = ymax;
    p.jre = jre;
    p.jim = jim;
    p.out = d_out;
    p.sync = (FrameSync*)ctx->sync.ptr;
    p.tile_rows_done = nullptr;
    p.band_flags = nullptr;
    p.stop = nullptr;
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
    if ((rc = launch_fp64(ctx, p, ctx->stream)))
        return rc;
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    int64_t d2h = 0;
    if (h_out) {
        MDZ_CUDA_TRY(cudaMemcpyAsync(h_out, d_out, n * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                     ctx->stream));
        d2h = (int64_t)(n * sizeof(int32_t));
    }
    return finish_stats(ctx, st, t0, 1, 0, d2h);
}

int mdzgpu_render_fp64(mdzgpu_ctx* ctx, const mdzgpu_frame* f, double xmin, double xmax,
                       double ymax, double julia_re, double julia_im, int32_t* counts,
                       mdzgpu_stats* st)
{
    if (!counts) {
        set_error("null counts buffer");
        return MDZGPU_ERR_ARG;
    }
    return fp64_common(ctx, f, xmin, xmax, ymax, julia_re, julia_im, nullptr, counts, st);
}

int mdzgpu_render_fp64_device(mdzgpu_ctx* ctx, const mdzgpu_frame* f, double xmin,
                              double xmax, double ymax, double julia_re, double julia_im,
                              int32_t* d_counts, mdzgpu_stats* st)
{
    if (!d_counts) {
        set_error("null device counts buffer");
        return MDZGPU_ERR_ARG;
    }
    return fp64_common(ctx, f, xmin, xmax, ymax, julia_re, julia_im, d_counts, nullptr, st);
}

int32_t mdzgpu_mp_max_words(void)
{
    int w = kMpThreadMaxWords;
#define MDZ_CASE(n, g, q) \
    if (n > w)            \
        w = n;
    MDZ_MPW_LIST(MDZ_CASE)
#undef MDZ_CASE
    return w;
}

static int pick_words(long precision, int words)
{
    if (words <= 0)
        words = mp_words_for_precision(precision);
    for (int w = words; w <= mdzgpu_mp_max_words(); ++w)
        if (mp_words_supported(w))
            return w;
    return -1;
}

// Builds the fixed-point x / y tables of a frame on the host:
//   x[ix]   = xmin + ix * width / W
//   y[line] = ymax - line * width / W
static int mp_tables(const uint32_t* xmin, const uint32_t* ymax, const uint32_t* width, int W,
                     int H, int words, std::vector<uint32_t>& tab)
{
    tab.assign((size_t)(W + H) * words, 0);
    for (int ix = 0; ix < W; ++ix) {
        uint32_t* o = &tab[(size_t)ix * words];
        fx_affine(xmin, width, ix, W, +1, words, o);
        if (!fx_fits_coordinate(o, words))
            return MDZGPU_ERR_RANGE;
    }
    for (int y = 0; y < H; ++y) {
        uint32_t* o = &tab[(size_t)(W + y) * words];
        fx_affine(ymax, width, y, W, -1, words, o);
        if (!fx_fits_coordinate(o, words))
            return MDZGPU_ERR_RANGE;
    }
    return MDZGPU_OK;
}

}  // extern "C"

namespace mdz {

int mp_render_tables(mdzgpu_ctx* ctx, const mdzgpu_frame* f, int words,
                     const std::vector<uint32_t>& tab, int32_t* d_out, int32_t* h_out,
                     mdzgpu_stats* st, double t0)
{
    int rc;
    const int W = f->width, H = f->height;
    const size_t n = (size_t)W * H;
    if (!d_out) {
        if ((rc = ctx->counts.ensure(n * sizeof(int32_t))))
            return rc;
        d_out = (int32_t*)ctx->counts.ptr;
    }
    if ((rc = ctx->sync.ensure(sizeof(FrameSync))) || (rc = ctx->coords.ensure(tab.size() * 4)))
        return rc;
    if (st)
        memset(st, 0, sizeof *st);
    MDZ_CUDA_TRY(cudaMemcpyAsync(ctx->coords.ptr, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice,
                                 ctx->stream));
    MDZ_CUDA_TRY(cudaMemsetAsync(ctx->sync.ptr, 0, sizeof(FrameSync), ctx->stream));
    MpLaunch p;
    p.W = W;
    p.H = H;
    p.row0 = 0;
    p.nrows = H;
    p.family = f->family;
    p.fractal = f->fractal;
    p.depth = (uint32_t)f->depth;
    p.words = words;
    p.xs = (const uint32_t*)ctx->coords.ptr;
    p.ys = p.xs + (size_t)W * words;
    p.julia = p.xs + (size_t)(W + H) * words;
    p.out = d_out;
    p.sync = (FrameSync*)ctx->sync.ptr;
    p.tile_rows_done = nullptr;
    p.band_flags = nullptr;
    p.stop = nullptr;
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
    if ((rc = launch_mp(ctx, p, ctx->stream)))
        return rc;
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    int64_t d2h = 0;
    if (h_out) {
        MDZ_CUDA_TRY(cudaMemcpyAsync(h_out, d_out, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
        d2h = (int64_t)n * 4;
    }
    rc = finish_stats(ctx, st, t0, 1, (int64_t)tab.size() * 4, d2h);
    if (st)
        st->words = words;
    return rc;
}

}  // namespace mdz

extern "C" {

static int mp_common(mdzgpu_ctx* ctx, const mdzgpu_frame* f, const mdzgpu_mpval* xmin,
                     const mdzgpu_mpval* ymax, const mdzgpu_mpval* width,
                     const mdzgpu_mpval* jre, const mdzgpu_mpval* jim, int64_t precision,
                     int32_t words, int32_t* d_out, int32_t* h_out, mdzgpu_stats* st)
{
    const double t0 = now_ms();
    if (!ctx) {
        set_error("null context");
        return MDZGPU_ERR_ARG;
    }
    int rc = validate_frame(f);
    if (rc)
        return rc;
    MDZ_CUDA_TRY(cudaSetDevice(ctx->device));
    const int w = pick_words((long)precision, words);
    if (w < 0) {
        set_error("precision %lld needs more than %d words", (long long)precision,
                  mdzgpu_mp_max_words());
        return MDZGPU_ERR_UNSUPPORTED;
    }
    // x[ix], y[line] and the julia constant exactly as MPFR computes them
    // at `precision` bits (src/fractal.c:159-203)
    const int W = f->width, H = f->height;
    std::vector<uint32_t> tab((size_t)(W + H + 2) * w, 0);
    int rc2 = mpfr_coordinate_tables(xmin, ymax, width, W, 0, H, (long)precision, w, tab.data(),
                                     tab.data() + (size_t)W * w);
    if (!rc2 && f->family == MDZ_FAMILY_JULIA)
        rc2 = mpfr_round_to_fixed(jre, (long)precision, w, tab.data() + (size_t)(W + H) * w)
              | mpfr_round_to_fixed(jim, (long)precision, w, tab.data() + (size_t)(W + H + 1) * w);
    if (rc2 || (f->family == MDZ_FAMILY_JULIA
                && (!fx_fits_coordinate(tab.data() + (size_t)(W + H) * w, w)
                    || !fx_fits_coordinate(tab.data() + (size_t)(W + H + 1) * w, w)))) {
        set_error("multi-limb path: coordinates must satisfy |x|, |y| < 4");
        return MDZGPU_ERR_RANGE;
    }
    return mp_render_tables(ctx, f, w, tab, d_out, h_out, st, t0);
}

int mdzgpu_render_mp(mdzgpu_ctx* ctx, const mdzgpu_frame* f, const mdzgpu_mpval* xmin,
                     const mdzgpu_mpval* ymax, const mdzgpu_mpval* width,
                     const mdzgpu_mpval* julia_re, const mdzgpu_mpval* julia_im,
                     int64_t precision, int32_t words, int32_t* counts, mdzgpu_stats* st)
{
    if (!counts) {
        set_error("null counts buffer");
        return MDZGPU_ERR_ARG;
    }
    return mp_common(ctx, f, xmin, ymax, width, julia_re, julia_im, precision, words, nullptr,
                     counts, st);
}

int mdzgpu_render_mp_device(mdzgpu_ctx* ctx, const mdzgpu_frame* f, const mdzgpu_mpval* xmin,
                            const mdzgpu_mpval* ymax, const mdzgpu_mpval* width,
                            const mdzgpu_mpval* julia_re, const mdzgpu_mpval* julia_im,
                            int64_t precision, int32_t words, int32_t* d_counts,
                            mdzgpu_stats* st)
{
    if (!d_counts) {
        set_error("null device counts buffer");
        return MDZGPU_ERR_ARG;
    }
    return mp_common(ctx, f, xmin, ymax, width, julia_re, julia_im, precision, words, d_counts,
                     nullptr, st);
}

int mdzgpu_mp_coordinates(const mdzgpu_mpval* xmin, const mdzgpu_mpval* ymax,
                          const mdzgpu_mpval* width, int32_t W, int32_t row0, int32_t nrows,
                          int64_t precision, int32_t words, uint32_t* xs, uint32_t* ys)
{
    if (!xs || !ys || W <= 0 || nrows < 0 || words < 4)
        return MDZGPU_ERR_ARG;
    return mpfr_coordinate_tables(xmin, ymax, width, W, row0, nrows, (long)precision, words, xs,
                                  ys);
}

int mdzgpu_fx_from_mpval(const mdzgpu_mpval* v, int32_t words, uint32_t* out)
{
    if (!out || words < 2)
        return MDZGPU_ERR_ARG;
    return fx_from_mpval(v, words, out);
}

int mdzgpu_perturb_spacing(const mdzgpu_mpval* width, int32_t W, double* hs_m, int32_t* hs_e)
{
    int e = 0;
    int rc = half_spacing(width, W, hs_m, &e);
    if (hs_e)
        *hs_e = e;
    return rc;
}

int mdzgpu_set_wait_limit(mdzgpu_ctx* ctx, int32_t polls)
{
    if (!ctx || polls < 0) {
        set_error("wait limit: null context or negative poll count");
        return MDZGPU_ERR_ARG;
    }
    ctx->wait_limit = polls ? polls : kSpinLimit;
    return MDZGPU_OK;
}

int32_t mdzgpu_perturb_limbs(int64_t precision)
{
    long L = (long)((precision + 27) / 28) + 1;
    if (L < 5)
        L = 5;
    return (int32_t)L;
}

// Bits a pass may lose to rebase cancellation before its pixel is re-run by
// the next, more precise pass (FP32 -> FP64 -> multi-limb).
constexpr float kLostLimitFp32 = 1.0f;
constexpr float kLostLimitFp64 = 6.0f;


// Fixed-point pixel coordinates of the perturbation geometry for the
// multi-limb pass: x[ix] = cx + (2 ix - W) hs, y[line] = cy + (H - 2 line) hs.
}  // extern "C"

namespace mdz {

OrbitLayout orbit_layout(size_t entries, int L)
{
    // zq[entries] float4 | zd[entries] double2 | ze[entries] int |
    // dd[entries] double | de[entries] int | tiny bits | fm[entries] double |
    // fe[entries] int | axis bits | attention bits | len + progress words |
    // centre digits | rebases | digits[entries][2][L] int (raw orbit, scratch)
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    OrbitLayout o;
    o.zd = al(entries * sizeof(float4));
    o.ze = o.zd + al(entries * sizeof(double2));
    o.dd = o.ze + al(entries * sizeof(int));
    o.de = o.dd + al(entries * sizeof(double));
    o.tiny = o.de + al(entries * sizeof(int));
    o.fm = o.tiny + al((entries / 32 + 40) * sizeof(unsigned));  // + whole last batches
    o.fe = o.fm + al(entries * sizeof(double));
    o.axis = o.fe + al(entries * sizeof(int));
    o.att = o.axis + al((entries / 32 + 40) * sizeof(unsigned));
    o.len = o.att + al((entries / 32 + 40) * sizeof(unsigned));
    o.dig = o.len + 256;
    o.reb = o.dig + al(2 * (size_t)L * sizeof(int));
    o.raw = o.reb + 256;
    o.bytes = o.raw + al(entries * 2 * (size_t)L * sizeof(int));
    return o;
}

int perturb_mp_words(long precision)
{
    const int words = mp_words_for_precision(precision);
    for (int k = words; k <= mdzgpu_mp_max_words(); ++k)
        if (mp_words_supported(k))
            return k;
    return mdzgpu_mp_max_words();
}

int perturb_tables(const mdzgpu_mpval* cx, const mdzgpu_mpval* cy, double hs_m, int hs_e,
                          int W, int H, int words, std::vector<uint32_t>& tab)
{
    std::vector<uint32_t> fcx(words), fcy(words), fhs(words);
    if (fx_from_mpval(cx, words, fcx.data()) || fx_from_mpval(cy, words, fcy.data()))
        return MDZGPU_ERR_RANGE;
    // hs = (hs_m 2^39) 2^(hs_e - 39), hs_m 2^39 an integer below 2^40
    const uint64_t hint = (uint64_t)ldexp(hs_m, 39);
    uint64_t limb[1] = {hint << 24};
    mdzgpu_mpval hv;
    hv.sign = 1;
    hv.nlimbs = 1;
    hv.exp = (int64_t)hs_e + 1;   // hint << 24 is normalised: 0.(hint<<24) 2^exp
    hv.d = limb;
    if (fx_from_mpval(&hv, words, fhs.data()))
        return MDZGPU_ERR_RANGE;
    for (int ix = 0; ix < W; ++ix) {
        const long k = 2L * ix - W;
        fx_affine(fcx.data(), fhs.data(), k < 0 ? -k : k, 1, k < 0 ? -1 : +1, words,
                  tab.data() + (size_t)ix * words);
        if (!fx_fits_coordinate(tab.data() + (size_t)ix * words, words))
            return MDZGPU_ERR_RANGE;
    }
    for (int y = 0; y < H; ++y) {
        const long k = (long)H - 2L * y;
        fx_affine(fcy.data(), fhs.data(), k < 0 ? -k : k, 1, k < 0 ? -1 : +1, words,
                  tab.data() + (size_t)(W + y) * words);
        if (!fx_fits_coordinate(tab.data() + (size_t)(W + y) * words, words))
            return MDZGPU_ERR_RANGE;
    }
    return MDZGPU_OK;
}

}  // namespace mdz

extern "C" {

// Pass 0 in steps while the streamed orbit (already launched on ctx->side,
// completion event `orbit_done_ev`) is produced.  Each step: every
// unfinished pixel runs at most `budget` iterations or up to the last
// finished orbit entry; the unfinished ones are compacted into the other
// queue.  The budget keeps one step near 8 ms of GPU time.
static int perturb_steps(mdzgpu_ctx* ctx, const PerturbLaunch& p, size_t n,
                         cudaEvent_t orbit_done_ev, int* launches, double* pixel_ms,
                         int64_t* pixel_launches)
{
    int rc;
    if ((rc = ctx->pstate.ensure(n * 32)) || (rc = ctx->pqueue.ensure(2 * n * 4 + 256))
        || (rc = ctx->stepinfo.ensure(256)))
        return rc;
    unsigned* counters = (unsigned*)ctx->pqueue.ptr;           // pull, count
    unsigned* qa = (unsigned*)((char*)ctx->pqueue.ptr + 256);
    unsigned* qb = qa + n;
    volatile unsigned* h_count = (volatile unsigned*)ctx->stepinfo.host;
    volatile int* h_orbit_err = (volatile int*)ctx->stepinfo.host + 1;
    const unsigned* in = nullptr;   // first step: every pixel, fresh
    unsigned* out = qa;
    unsigned left = (unsigned)n;
    bool orbit_finished = false;
    // a pixel stops at least every `budget` iterations, or when it waits for
    // the orbit: after the orbit is complete every step advances every
    // pixel, so the loop ends within depth / budget_min steps of it
    const double rate = 3.0e11;       // pixel-iterations/s of the FP32 pass
    for (long step = 0;; ++step) {
        const double b = rate * 8e-3 / (double)left;
        const unsigned budget = (unsigned)std::min(std::max(b, 256.0), (double)(1u << 24));
        if ((rc = launch_perturb_step(ctx->num_sms, p, in, left, out, counters,
                                      (uint4*)ctx->pstate.ptr, budget, ctx->stream, ctx->ev_k0,
                                      ctx->ev_k1)))
            return rc;
        MDZ_CUDA_TRY(cudaMemcpyAsync((void*)h_count, counters + 1, 4, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        float kms = 0.f;
        MDZ_CUDA_TRY(cudaEventElapsedTime(&kms, ctx->ev_k0, ctx->ev_k1));
        *pixel_ms += kms;
        ++*pixel_launches;
        *launches += 2;
        left = *h_count;
        if (left == 0)
            return MDZGPU_OK;
        in = out;
        out = (out == qa) ? qb : qa;
        if (!orbit_finished) {
            const cudaError_t e = cudaEventQuery(orbit_done_ev);
            if (e == cudaSuccess) {
                orbit_finished = true;
                MDZ_CUDA_TRY(cudaMemcpyAsync((void*)h_orbit_err, p.orbit_error, 4,
                                             cudaMemcpyDeviceToHost, ctx->side));
                MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->side));
                if (*h_orbit_err) {
                    set_error("perturbation: a bounded wait of the orbit finisher gave up");
                    return MDZGPU_ERR_TIMEOUT;
                }
            } else if (e != cudaErrorNotReady) {
                MDZ_CUDA_TRY(e);
            }
        }
    }
}

// jre / jim: the Julia constant (Julia family), else null.
static int perturb_common(mdzgpu_ctx* ctx, const mdzgpu_frame* f, const mdzgpu_mpval* cx,
                          const mdzgpu_mpval* cy, const mdzgpu_mpval* width, int64_t precision,
                          int32_t limbs, int32_t* d_out, float* d_mag, int32_t* h_out,
                          float* h_mag, mdzgpu_stats* st, const mdzgpu_mpval* jre = nullptr,
                          const mdzgpu_mpval* jim = nullptr)
{
    const double t0 = now_ms();
    if (!ctx) {
        set_error("null context");
        return MDZGPU_ERR_ARG;
    }
    int rc = validate_frame(f);
    if (rc)
        return rc;
    const bool julia = f->family == MDZ_FAMILY_JULIA;
    const bool variant = f->fractal == MDZ_VARIANT;
    if ((f->family != MDZ_FAMILY_MANDEL && !julia) || (julia && variant)) {
        set_error("perturbation: the Mandelbrot family with any formula, or the Julia family "
                  "with the Mandelbrot, burning ship or celtic formula");
        return MDZGPU_ERR_UNSUPPORTED;
    }
    if (julia != (jre && jim)) {
        set_error(julia ? "perturbation: the Julia family needs its constant"
                        : "perturbation: a Julia constant outside the Julia family");
        return MDZGPU_ERR_ARG;
    }
    MDZ_CUDA_TRY(cudaSetDevice(ctx->device));
    const int L = limbs > 0 ? limbs : mdzgpu_perturb_limbs(precision);
    if (L > orbit_max_limbs() || L < 5) {
        set_error("perturbation: %d orbit limbs outside [5, %d]", L, orbit_max_limbs());
        return MDZGPU_ERR_UNSUPPORTED;
    }
    // digits: the centre, then (Julia) the constant
    std::vector<int> dig((julia ? 4 : 2) * (size_t)L);
    if (digits28_from_mpval(cx, L, dig.data()) || digits28_from_mpval(cy, L, dig.data() + L)) {
        set_error("perturbation: centre outside the fixed-point range");
        return MDZGPU_ERR_RANGE;
    }
    if (abs(dig[L - 1]) >= 4 || abs(dig[2 * L - 1]) >= 4) {
        set_error("perturbation: centre must satisfy |cx|, |cy| < 4");
        return MDZGPU_ERR_RANGE;
    }
    if (julia && (digits28_from_mpval(jre, L, dig.data() + 2 * L)
                  || digits28_from_mpval(jim, L, dig.data() + 3 * L)
                  || abs(dig[3 * L - 1]) >= 4 || abs(dig[4 * L - 1]) >= 4)) {
        set_error("perturbation: the Julia constant must satisfy |re|, |im| < 4");
        return MDZGPU_ERR_RANGE;
    }
    double hs_m = 0.0;
    int hs_e = 0;
    if ((rc = half_spacing(width, f->width, &hs_m, &hs_e)))
        return rc;
    const size_t n = (size_t)f->width * f->height;
    // Julia: the view orbit V in entries [0, q0), the critical orbit Q from
    // q0 (a multiple of 1024, so both bit masks start on a word); the
    // hybrid: the orbits that fold at odd / even steps
    const bool two = julia || variant;
    const size_t q0 = two ? ((size_t)f->depth + 2 + 1023) / 1024 * 1024 : 0;
    const OrbitLayout ol = orbit_layout(q0 + (size_t)f->depth + 2, L);
    const size_t off_zd = ol.zd, off_ze = ol.ze, off_dd = ol.dd, off_de = ol.de;
    const size_t off_len = ol.len, off_dig = ol.bytes, off_reb = ol.reb, off_raw = ol.raw;
    const size_t orbit_bytes = ol.bytes + dig.size() * sizeof(int);
    if ((rc = ctx->orbit.ensure(orbit_bytes)) || (rc = ctx->sync.ensure(sizeof(FrameSync))))
        return rc;
    if (!d_out) {
        if ((rc = ctx->counts.ensure(n * sizeof(int32_t))))
            return rc;
        d_out = (int32_t*)ctx->counts.ptr;
    }
    if (!d_mag && h_mag) {
        if ((rc = ctx->aux.ensure(n * sizeof(float))))
            return rc;
        d_mag = (float*)ctx->aux.ptr;
    }
    if (st)
        memset(st, 0, sizeof *st);
    char* ob = (char*)ctx->orbit.ptr;
    MDZ_CUDA_TRY(cudaMemcpyAsync(ob + off_dig, dig.data(), dig.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, ctx->stream));
    MDZ_CUDA_TRY(cudaMemsetAsync(ob + off_reb, 0, 256, ctx->stream));
    MDZ_CUDA_TRY(cudaMemsetAsync(ctx->sync.ptr, 0, sizeof(FrameSync), ctx->stream));
    OrbitLaunch o;
    o.limbs = L;
    o.c_re = (const int*)(ob + off_dig);
    o.c_im = o.c_re + L;
    o.zq = (float4*)ob;
    o.zd = (double2*)(ob + off_zd);
    o.ze = (int*)(ob + off_ze);
    o.dd = (double*)(ob + off_dd);
    o.de = (int*)(ob + off_de);
    o.digits = (int*)(ob + off_raw);
    o.max_k = (int)f->depth + 1;
    o.out_len = (int*)(ob + off_len);
    o.tiny = (unsigned*)(ob + ol.tiny);
    o.fractal = f->fractal;
    o.fm = (double*)(ob + ol.fm);
    o.fe = (int*)(ob + ol.fe);
    o.axis = (unsigned*)(ob + ol.axis);
    o.att = (unsigned*)(ob + ol.att);
    o.spin_limit = ctx->wait_limit;
    OrbitLaunch oq = o;   // Julia: the critical orbit; hybrid: the even-step one
    if (two) {
        if (julia) {
            // V: Z_0 = centre, constant c_J; Q: Z_0 = 0, constant c_J
            o.z0_re = o.c_re;
            o.z0_im = o.c_im;
            o.c_re = o.c_re + 2 * L;
            o.c_im = o.c_re + L;
            oq.c_re = o.c_re;
            oq.c_im = o.c_im;
        } else {
            o.fold_parity = 1;
            oq.fold_parity = 0;
        }
        oq.zq = o.zq + q0;
        oq.zd = o.zd + q0;
        oq.ze = o.ze + q0;
        oq.dd = o.dd + q0;
        oq.de = o.de + q0;
        oq.fm = o.fm + q0;
        oq.fe = o.fe + q0;
        oq.tiny = o.tiny + q0 / 32;
        oq.axis = o.axis + q0 / 32;
        oq.att = o.att + q0 / 32;
        oq.out_len = o.out_len + 16;   // beside V's length, in the zeroed progress block
    }
    int64_t h2d_extra = 0;
    cudaEvent_t evo;
    MDZ_CUDA_TRY(cudaEventCreate(&evo));
    // progress words of the fused launch live beside out_len
    int* prog = (int*)(ob + off_len);
    MDZ_CUDA_TRY(cudaMemsetAsync(prog, 0, 256, ctx->stream));
    // Pass 0 schedule (MDZGPU_PERTURB):
    //   "steps" (default): the orbit runs as a cooperative producer/finisher
    //     launch on the side stream while the frame's pixels iterate in
    //     steps on the main stream; a step lets every unfinished pixel run
    //     until its budget or the last finished orbit entry, then compacts
    //     the unfinished pixels; the orbit's serial time hides behind the
    //     pixel work;
    //   "frame": the orbit first, then one launch over the whole frame;
    //   "fused": orbit and pixels in one cooperative grid (slower: the
    //     resident first wave is paced by the orbit).
    const char* menv = getenv("MDZGPU_PERTURB");
    const char* fenv = getenv("MDZGPU_FUSED");
    const bool fused = ((fenv && fenv[0] == '1') || (menv && !strcmp(menv, "fused")))
                       && f->fractal == MDZ_MANDELBROT && !two;
    // two orbits: both first (every rebase may need any entry of either)
    const bool stepped = !fused && !two && !(menv && !strcmp(menv, "frame"));
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
    if (stepped) {
        MDZ_CUDA_TRY(cudaEventRecord(evo, ctx->stream));   // inputs in place
        MDZ_CUDA_TRY(cudaStreamWaitEvent(ctx->side, evo, 0));
        MDZ_CUDA_TRY(cudaEventRecord(ctx->ev_side0, ctx->side));
        if ((rc = launch_orbit_stream(o, prog, ctx->side))) {
            cudaEventDestroy(evo);
            return rc;
        }
        MDZ_CUDA_TRY(cudaEventRecord(evo, ctx->side));      // orbit complete
    } else {
        if (!fused) {
            if ((rc = launch_orbit(o, ctx->stream))
                || (two && (rc = launch_orbit(oq, ctx->stream)))) {
                cudaEventDestroy(evo);
                return rc;
            }
        }
        MDZ_CUDA_TRY(cudaEventRecord(evo, ctx->stream));
    }
    PerturbLaunch p;
    p.W = f->width;
    p.H = f->height;
    p.row0 = 0;
    p.nrows = f->height;
    p.depth = (uint32_t)f->depth;
    p.hs_m = hs_m;
    p.hs_e = hs_e;
    p.zq = o.zq;
    p.zd = o.zd;
    p.ze = o.ze;
    p.dd = o.dd;
    p.de = o.de;
    p.orbit_len = o.out_len;
    p.tiny = o.tiny;
    p.att = o.att;
    p.fractal = f->fractal;
    p.fm = o.fm;
    p.fe = o.fe;
    p.axis = o.axis;
    if (two) {
        p.q0 = (int)q0;
        p.q_len = oq.out_len;
        p.julia = julia;
    }
    p.out = d_out;
    p.mag = d_mag;
    p.sync = (FrameSync*)ctx->sync.ptr;
    p.rebases = (unsigned long long*)(ob + off_reb);
    p.stop = nullptr;
    p.spin_limit = ctx->wait_limit;
    // escalation lists: [count1 | count2 | pad] list1[n] list2[n]
    ctx->esc_pixels = 0;
    if ((rc = ctx->lists.ensure(256 + 2 * n * sizeof(unsigned)))) {
        cudaEventDestroy(evo);
        return rc;
    }
    unsigned* counts_dev = (unsigned*)ctx->lists.ptr;
    unsigned* list1 = (unsigned*)((char*)ctx->lists.ptr + 256);
    unsigned* list2 = list1 + n;
    MDZ_CUDA_TRY(cudaMemsetAsync(ctx->lists.ptr, 0, 256, ctx->stream));
    // pass 0: FP32 mantissas over the frame (fused with the orbit when
    // MDZGPU_FUSED=1)
    p.lost_limit = kLostLimitFp32;
    p.flag_out = list1;
    p.flag_out_count = counts_dev;
    p.raw_len = prog + 1;
    p.fin_len = prog + 2;
    p.orbit_done = prog + 3;
    p.orbit_error = prog + 4;
    p.producer_sm = prog + 5;
    int launches = 5;
    double pixel_ms = 0.0;
    int64_t pixel_launches = 0;
    if (stepped) {
        rc = perturb_steps(ctx, p, n, evo, &launches, &pixel_ms, &pixel_launches);
        // the list passes read the whole orbit
        if (!rc && cudaStreamWaitEvent(ctx->stream, evo, 0) != cudaSuccess)
            rc = MDZGPU_ERR_CUDA;
    } else {
        rc = fused ? launch_fused(ctx, o, p, ctx->stream) : launch_perturb(ctx, p, ctx->stream, 0);
    }
    if (rc) {
        cudaEventDestroy(evo);
        return rc;
    }
    // pass 1: FP64 mantissas over the pixels pass 0 flagged
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev_k0, ctx->stream));
    MDZ_CUDA_TRY(cudaMemsetAsync(&((FrameSync*)ctx->sync.ptr)->tile_counter, 0, sizeof(unsigned),
                                 ctx->stream));
    p.list_in = list1;
    p.list_in_count = counts_dev;
    p.lost_limit = kLostLimitFp64;
    p.flag_out = list2;
    p.flag_out_count = counts_dev + 1;
    if ((rc = launch_perturb(ctx, p, ctx->stream, 1))) {
        cudaEventDestroy(evo);
        return rc;
    }
    // pass 2: the exact multi-limb kernel for what FP64 could not settle
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev_k1, ctx->stream));
    bool mp_skipped = false;
    {
        unsigned n_mp = 0;
        MDZ_CUDA_TRY(cudaMemcpyAsync(&n_mp, counts_dev + 1, 4, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        // (Routing a short list at 28-36 words to the warp-cooperative kernel
        // at 48 words was measured slower: 13190 pixels at depth 51503,
        // 385 -> 1593 ms; 3086 pixels at depth 200000, 2083 -> 2851 ms.)
        const int w = perturb_mp_words((long)precision);
        std::vector<uint32_t> tab((size_t)(f->width + f->height + 2) * w, 0);
        if ((rc = perturb_tables(cx, cy, hs_m, hs_e, f->width, f->height, w, tab))
            || (julia
                && (fx_from_mpval(jre, w, tab.data() + (size_t)(f->width + f->height) * w)
                    || fx_from_mpval(jim, w, tab.data() + (size_t)(f->width + f->height + 1) * w)))) {
            set_error("perturbation: coordinates outside the fixed-point range");
            cudaEventDestroy(evo);
            return rc ? rc : MDZGPU_ERR_RANGE;
        }
        mp_skipped = n_mp == 0;
        if (n_mp == 0) {
            --launches;   // nothing left for the multi-limb kernel
        } else {
            if ((rc = ctx->coords.ensure(tab.size() * 4))) {
                cudaEventDestroy(evo);
                return rc;
            }
            MDZ_CUDA_TRY(cudaMemcpyAsync(ctx->coords.ptr, tab.data(), tab.size() * 4,
                                         cudaMemcpyHostToDevice, ctx->stream));
            MDZ_CUDA_TRY(cudaMemsetAsync(&((FrameSync*)ctx->sync.ptr)->tile_counter, 0,
                                         sizeof(unsigned), ctx->stream));
            MpLaunch q;
            q.W = f->width;
            q.H = f->height;
            q.row0 = 0;
            q.nrows = f->height;
            q.family = julia ? MDZ_FAMILY_JULIA : MDZ_FAMILY_MANDEL;
            q.fractal = f->fractal;
            q.depth = (uint32_t)f->depth;
            q.words = w;
            q.xs = (const uint32_t*)ctx->coords.ptr;
            q.ys = q.xs + (size_t)f->width * w;
            q.julia = q.xs + (size_t)(f->width + f->height) * w;
            q.out = d_out;
            q.sync = (FrameSync*)ctx->sync.ptr;
            q.tile_rows_done = nullptr;
            q.band_flags = nullptr;
            q.stop = nullptr;
            q.list = list2;
            q.list_count = counts_dev + 1;
            q.mag = d_mag;
            if ((rc = launch_mp(ctx, q, ctx->stream))) {
                cudaEventDestroy(evo);
                return rc;
            }
            h2d_extra = (int64_t)tab.size() * 4;
        }
    }
    MDZ_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    int64_t d2h = 0;
    if (h_out) {
        MDZ_CUDA_TRY(cudaMemcpyAsync(h_out, d_out, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
        d2h += (int64_t)n * 4;
    }
    if (h_mag) {
        MDZ_CUDA_TRY(cudaMemcpyAsync(h_mag, d_mag, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
        d2h += (int64_t)n * 4;
    }
    unsigned long long reb = 0;
    int olen = 0;
    int orbit_err = 0;
    unsigned esc[2] = {0, 0};
    MDZ_CUDA_TRY(cudaMemcpyAsync(&orbit_err, prog + 4, 4, cudaMemcpyDeviceToHost, ctx->stream));
    MDZ_CUDA_TRY(cudaMemcpyAsync(esc, counts_dev, 8, cudaMemcpyDeviceToHost, ctx->stream));
    MDZ_CUDA_TRY(cudaMemcpyAsync(&reb, p.rebases, 8, cudaMemcpyDeviceToHost, ctx->stream));
    MDZ_CUDA_TRY(cudaMemcpyAsync(&olen, o.out_len, 4, cudaMemcpyDeviceToHost, ctx->stream));
    rc = finish_stats(ctx, st, t0, launches, (int64_t)dig.size() * 4 + h2d_extra, d2h + 20);
    if (!rc && orbit_err) {
        set_error("perturbation: a bounded wait on the reference orbit gave up");
        rc = MDZGPU_ERR_TIMEOUT;
    }
    if (!rc && st) {
        st->escalated_fp64 = esc[0];
        st->escalated_mp = esc[1];
        float oms = 0.f;
        cudaEventElapsedTime(&oms, stepped ? ctx->ev_side0 : ctx->ev0, evo);
        // fused: the orbit runs inside the pixel kernel and has no own time
        st->orbit_ms = fused ? -1.0 : oms;
        st->rebases = (int64_t)reb;
        st->orbit_len = olen;
        st->pixel_ms = pixel_ms;
        st->pixel_launches = pixel_launches;
        float e64 = 0.f, emp = 0.f;
        cudaEventElapsedTime(&e64, ctx->ev_k0, ctx->ev_k1);
        cudaEventElapsedTime(&emp, ctx->ev_k1, ctx->ev1);
        st->esc_fp64_ms = e64;
        st->esc_mp_ms = mp_skipped ? 0.0 : emp;
    }
    if (!rc)
        ctx->esc_pixels = (int64_t)n;
    cudaEventDestroy(evo);
    return rc;
}

int mdzgpu_last_escalations(mdzgpu_ctx* ctx, uint32_t* fp64, int64_t cap_fp64, int64_t* n_fp64,
                            uint32_t* mp, int64_t cap_mp, int64_t* n_mp)
{
    if (!ctx || !n_fp64 || !n_mp || cap_fp64 < 0 || cap_mp < 0 || (cap_fp64 && !fp64)
        || (cap_mp && !mp)) {
        set_error("escalations: null argument or negative capacity");
        return MDZGPU_ERR_ARG;
    }
    if (!ctx->esc_pixels) {
        set_error("escalations: no perturbation render on this context");
        return MDZGPU_ERR_ARG;
    }
    const int64_t n = ctx->esc_pixels;
    unsigned cnt[2] = {0, 0};
    MDZ_CUDA_TRY(cudaMemcpyAsync(cnt, ctx->lists.ptr, 8, cudaMemcpyDeviceToHost, ctx->stream));
    MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    const unsigned* list1 = (const unsigned*)((const char*)ctx->lists.ptr + 256);
    const int64_t k1 = std::min<int64_t>(cnt[0], cap_fp64), k2 = std::min<int64_t>(cnt[1], cap_mp);
    if (k1)
        MDZ_CUDA_TRY(cudaMemcpyAsync(fp64, list1, k1 * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (k2)
        MDZ_CUDA_TRY(cudaMemcpyAsync(mp, list1 + n, k2 * 4, cudaMemcpyDeviceToHost, ctx->stream));
    MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *n_fp64 = cnt[0];
    *n_mp = cnt[1];
    return MDZGPU_OK;
}

int mdzgpu_reference_orbit(mdzgpu_ctx* ctx, const mdzgpu_mpval* cx, const mdzgpu_mpval* cy,
                           int64_t precision, int32_t limbs, int64_t max_k, double* z_re,
                           double* z_im, double* d_mant, int32_t* d_exp, int64_t* len)
{
    return mdzgpu_reference_orbit_formula(ctx, MDZ_MANDELBROT, cx, cy, precision, limbs, max_k,
                                          z_re, z_im, d_mant, d_exp, len);
}

int mdzgpu_reference_orbit_formula(mdzgpu_ctx* ctx, int32_t fractal, const mdzgpu_mpval* cx,
                                   const mdzgpu_mpval* cy, int64_t precision, int32_t limbs,
                                   int64_t max_k, double* z_re, double* z_im, double* d_mant,
                                   int32_t* d_exp, int64_t* len)
{
    if (fractal < MDZ_MANDELBROT || fractal > MDZ_GENERALIZED_CELTIC) {
        set_error("reference orbit: formula %d has no multi-limb orbit", fractal);
        return MDZGPU_ERR_UNSUPPORTED;
    }
    if (!ctx || max_k < 1 || max_k > 0x7ffffffeLL) {
        set_error("reference orbit: bad arguments");
        return MDZGPU_ERR_ARG;
    }
    MDZ_CUDA_TRY(cudaSetDevice(ctx->device));
    const int L = limbs > 0 ? limbs : mdzgpu_perturb_limbs(precision);
    if (L > orbit_max_limbs() || L < 5) {
        set_error("reference orbit: %d limbs outside [5, %d]", L, orbit_max_limbs());
        return MDZGPU_ERR_UNSUPPORTED;
    }
    std::vector<int> dig(2 * (size_t)L);
    if (digits28_from_mpval(cx, L, dig.data()) || digits28_from_mpval(cy, L, dig.data() + L)) {
        set_error("reference orbit: centre outside the fixed-point range");
        return MDZGPU_ERR_RANGE;
    }
    const size_t entries = (size_t)max_k + 1;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t off_zd = al(entries * sizeof(float4));
    const size_t off_ze = off_zd + al(entries * sizeof(double2));
    const size_t off_dd = off_ze + al(entries * sizeof(int));
    const size_t off_de = off_dd + al(entries * sizeof(double));
    const size_t off_len = off_de + al(entries * sizeof(int));
    const size_t off_dig = off_len + 256;
    const size_t off_raw = off_dig + al(2 * L * sizeof(int));
    const size_t bytes = off_raw + al(entries * 2 * (size_t)L * sizeof(int));
    int rc = ctx->orbit.ensure(bytes);
    if (rc)
        return rc;
    char* ob = (char*)ctx->orbit.ptr;
    MDZ_CUDA_TRY(cudaMemcpyAsync(ob + off_dig, dig.data(), dig.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, ctx->stream));
    OrbitLaunch o;
    o.limbs = L;
    o.c_re = (const int*)(ob + off_dig);
    o.c_im = o.c_re + L;
    o.zq = (float4*)ob;
    o.zd = (double2*)(ob + off_zd);
    o.ze = (int*)(ob + off_ze);
    o.dd = (double*)(ob + off_dd);
    o.de = (int*)(ob + off_de);
    o.digits = (int*)(ob + off_raw);
    o.max_k = (int)max_k;
    o.out_len = (int*)(ob + off_len);
    o.fractal = fractal;
    if ((rc = launch_orbit(o, ctx->stream)))
        return rc;
    int n = 0;
    MDZ_CUDA_TRY(cudaMemcpyAsync(&n, o.out_len, 4, cudaMemcpyDeviceToHost, ctx->stream));
    MDZ_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    std::vector<double2> zd(n);
    std::vector<int> ze(n), de(n);
    std::vector<double> dd(n);
    MDZ_CUDA_TRY(cudaMemcpy(zd.data(), o.zd, n * sizeof(double2), cudaMemcpyDeviceToHost));
    MDZ_CUDA_TRY(cudaMemcpy(ze.data(), o.ze, n * sizeof(int), cudaMemcpyDeviceToHost));
    MDZ_CUDA_TRY(cudaMemcpy(dd.data(), o.dd, n * sizeof(double), cudaMemcpyDeviceToHost));
    MDZ_CUDA_TRY(cudaMemcpy(de.data(), o.de, n * sizeof(int), cudaMemcpyDeviceToHost));
    for (int k = 0; k < n; ++k) {
        if (z_re)
            z_re[k] = ldexp(zd[k].x, ze[k]);
        if (z_im)
            z_im[k] = ldexp(zd[k].y, ze[k]);
        if (d_mant)
            d_mant[k] = dd[k];
        if (d_exp)
            d_exp[k] = de[k];
    }
    if (len)
        *len = n;
    return MDZGPU_OK;
}

int mdzgpu_render_perturb(mdzgpu_ctx* ctx, const mdzgpu_frame* f, const mdzgpu_mpval* cx,
                          const mdzgpu_mpval* cy, const mdzgpu_mpval* width, int64_t precision,
                          int32_t limbs, int32_t* counts, float* mag2, mdzgpu_stats* st)
{
    if (!counts) {
        set_error("null counts buffer");
        return MDZGPU_ERR_ARG;
    }
    return perturb_common(ctx, f, cx, cy, width, precision, limbs, nullptr, nullptr, counts, mag2,
                          st);
}

int mdzgpu_render_perturb_julia(mdzgpu_ctx* ctx, const mdzgpu_frame* f, const mdzgpu_mpval* cx,
                                const mdzgpu_mpval* cy, const mdzgpu_mpval* width,
                                const mdzgpu_mpval* julia_re, const mdzgpu_mpval* julia_im,
                                int64_t precision, int32_t limbs, int32_t* counts, float* mag2,
                                mdzgpu_stats* st)
{
    if (!counts || !julia_re || !julia_im) {
        set_error("null argument");
        return MDZGPU_ERR_ARG;
    }
    return perturb_common(ctx, f, cx, cy, width, precision, limbs, nullptr, nullptr, counts, mag2,
                          st, julia_re, julia_im);
}

int mdzgpu_render_perturb_device(mdzgpu_ctx* ctx, const mdzgpu_frame* f,
                                 const mdzgpu_mpval* cx, const mdzgpu_mpval* cy,
                                 const mdzgpu_mpval* width, int64_t precision, int32_t limbs,
                                 int32_t* d_counts, float* d_mag2, mdzgpu_stats* st)
{
    if (!d_counts) {
        set_error("null device counts buffer");
        return MDZGPU_ERR_ARG;
    }
    return perturb_common(ctx, f, cx, cy, width, precision, limbs, d_counts, d_mag2, nullptr,
                          nullptr, st);
}

int mdzgpu_abi_layout(int64_t* out, int n)
{
    const int64_t offs[] = {
        (int64_t)offsetof(mdz_image_info, xmin),        (int64_t)offsetof(mdz_image_info, xmax),
        (int64_t)offsetof(mdz_image_info, ymax),        (int64_t)offsetof(mdz_image_info, width),
        (int64_t)offsetof(mdz_image_info, gxmin),       (int64_t)offsetof(mdz_image_info, gxmax),
        (int64_t)offsetof(mdz_image_info, gymax),       (int64_t)offsetof(mdz_image_info, gwidth),
        (int64_t)offsetof(mdz_image_info, old_cx),      (int64_t)offsetof(mdz_image_info, old_cy),
        (int64_t)offsetof(mdz_image_info, old_size),    (int64_t)offsetof(mdz_image_info, pcoords),
        (int64_t)offsetof(mdz_image_info, depth),       (int64_t)offsetof(mdz_image_info, thread_count),
        (int64_t)offsetof(mdz_image_info, draw_lines),  (int64_t)offsetof(mdz_image_info, raw_data),
        (int64_t)offsetof(mdz_image_info, rgb_data),    (int64_t)offsetof(mdz_image_info, j_pre),
        (int64_t)offsetof(mdz_image_info, drawing_area), (int64_t)offsetof(mdz_image_info, rnd_pal),
        (int64_t)offsetof(mdz_image_info, real_width),  (int64_t)offsetof(mdz_image_info, real_height),
        (int64_t)offsetof(mdz_image_info, user_width),  (int64_t)offsetof(mdz_image_info, user_height),
        (int64_t)offsetof(mdz_image_info, aspect),      (int64_t)offsetof(mdz_image_info, aa_factor),
        (int64_t)offsetof(mdz_image_info, family),      (int64_t)offsetof(mdz_image_info, fractal),
        (int64_t)offsetof(mdz_image_info, colour_scale), (int64_t)offsetof(mdz_image_info, u.julia.c_re),
        (int64_t)offsetof(mdz_image_info, u.julia.c_im), (int64_t)offsetof(mdz_image_info, palette_ip),
        (int64_t)offsetof(mdz_image_info, zoom_new_win), (int64_t)offsetof(mdz_image_info, use_multi_prec),
        (int64_t)offsetof(mdz_image_info, use_rounding), (int64_t)offsetof(mdz_image_info, precision),
        (int64_t)offsetof(mdz_image_info, multi_prec_init_done), (int64_t)offsetof(mdz_image_info, rth_ptr),
        (int64_t)offsetof(mdz_image_info, lines_drawn), (int64_t)offsetof(mdz_image_info, ui_ref_center),
        (int64_t)sizeof(mdz_image_info),
        (int64_t)offsetof(mdz_rthdata, img),            (int64_t)offsetof(mdz_rthdata, lines_drawn),
        (int64_t)offsetof(mdz_rthdata, min_line_drawn), (int64_t)offsetof(mdz_rthdata, line_draw_count),
        (int64_t)offsetof(mdz_rthdata, thread_count),   (int64_t)offsetof(mdz_rthdata, check_stop_px),
        (int64_t)offsetof(mdz_rthdata, data),           (int64_t)sizeof(mdz_rthdata),
    };
    const int cnt = (int)(sizeof offs / sizeof offs[0]);
    int k = 0;
    for (; k < cnt && k < n; ++k)
        out[k] = offs[k];
    return k;
}

}  // extern "C"
