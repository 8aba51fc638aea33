// Drop-in replacement for MDZ's render_threads.c + fractal.c entry points.
//
// Public behaviour kept from the reference (src/render_threads.c):
//   - rth_create / rth_init / rth_ui_init / rth_ui_start_render /
//     rth_ui_stop_render / rth_ui_stop_render_and_wait / rth_ui_quit /
//     rth_ui_wait_until_started / rth_ui_get_render_time /
//     rth_set_next_line_cb / rth_process_lines_rendered /
//     rth_render_should_stop / rth_ui_wait_for_line_done, with the same
//     return conventions and the same lines_rendered (0 -> 1 -> 2) /
//     lines_drawn / min_line_* progress protocol that render.c:49-92 and the
//     GUI's idle callback consume;
//   - a watch thread waiting for start requests and a render thread per
//     render (src/render_threads.c:185-339);
//   - the status word RT_STOP / RT_QUIT / RT_RENDERING (:9-14).
// What changes: the render thread does not spawn row workers.  It launches
// ONE kernel over the whole frame (method chosen by the installed callback)
// that pulls tiles from a device work counter and raises host-mapped flags
// as 4-row bands complete; the render thread turns those flags into
// lines_rendered[] updates and lines_rendered_cond signals, copying finished
// rows from pinned staging into img->raw_data.  Stop requests reach the
// kernel through a host-mapped stop word polled once per tile (the analogue
// of check_stop_px, src/fractal.c:113).
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>
#include <unistd.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "internal.h"

using namespace mdz;

namespace {

enum { RT_STOP = 0x0002, RT_QUIT = 0x0004, RT_RENDERING = 0x0008 };

enum Method { M_FP64, M_MPFR, M_GMP, M_HOST };

}  // namespace

struct mdz_rth_private {
    bool initialized = false;
    int thread_count = 0;
    char* lines_rendered = nullptr;
    int min_line_rendered = 0;
    int total_lines_rendered = 0;
    int (*next_line_cb)(mdz_image_info*, int) = nullptr;
    int start = 0;
    int started = 0;
    int status = 0;
    pthread_t watch_thread{};
    pthread_t render_thread{};
    bool watch_live = false;
    bool render_live = false;
    pthread_mutex_t start_mutex, started_mutex, status_mutex, lines_mutex;
    pthread_cond_t start_cond, started_cond, lines_cond;
    struct timeval tv_start {}, tv_end {};
    mdzgpu_ctx* ctx = nullptr;
};

namespace {

int get_status(mdz_rth_private* d)
{
    pthread_mutex_lock(&d->status_mutex);
    int s = d->status;
    pthread_mutex_unlock(&d->status_mutex);
    return s;
}

void set_status(mdz_rth_private* d, int s)
{
    pthread_mutex_lock(&d->status_mutex);
    d->status = s;
    pthread_mutex_unlock(&d->status_mutex);
}

// Publish user row `y` (its aa real rows are in raw_data).
void publish_row(mdz_rthdata* rth, int y)
{
    mdz_rth_private* d = rth->data;
    pthread_mutex_lock(&d->lines_mutex);
    d->lines_rendered[y] = 1;
    d->total_lines_rendered += rth->img->aa_factor;
    pthread_cond_signal(&d->lines_cond);
    pthread_mutex_unlock(&d->lines_mutex);
}

// On a failure the caller must still see the render finish (render.c waits
// for every row): report the error and publish the remaining rows.
void fail_remaining(mdz_rthdata* rth, const std::vector<char>& row_done)
{
    fprintf(stderr, "mdzgpu: render failed: %s\n", mdzgpu_last_error());
    for (int y = 0; y < rth->img->user_height; ++y)
        if (!row_done[y])
            publish_row(rth, y);
}

Method classify(int (*cb)(mdz_image_info*, int))
{
    if (cb == fractal_calculate_line)
        return M_FP64;
    if (cb == fractal_mpfr_calculate_line)
        return M_MPFR;
    if (cb == fractal_gmp_calculate_line)
        return M_GMP;
    return M_HOST;
}

int device_index()
{
    const char* s = getenv("MDZGPU_DEVICE");
    return s ? atoi(s) : 0;
}

mdzgpu_mpval as_mpval(const mdz_mpfr* v)
{
    mdzgpu_mpval m;
    m.sign = v->sign < 0 ? -1 : 1;
    m.exp = v->exp;
    m.nlimbs = v->exp == MDZ_MPFR_EXP_ZERO ? 0 : (int32_t)((v->prec + 63) / 64);
    m.d = m.nlimbs ? v->d : nullptr;
    return m;
}

// Fixed-point tables for rows [row0, row0 + nrows): x[W] | y[nrows] |
// julia c_re | c_im.  MPFR callback: MPFR's own p-bit coordinate roundings
// (src/fractal.c:159-203).  GMP callback: exact values from gxmin / gymax /
// gwidth (src/fractal.c:299-332 reads those).
bool frame_tables(const mdz_image_info* img, Method method, int words, int row0, int nrows,
                  std::vector<uint32_t>& tab)
{
    const int W = img->real_width;
    uint32_t* xs = tab.data();
    uint32_t* ys = xs + (size_t)W * words;
    uint32_t* jc = ys + (size_t)nrows * words;
    int rc = 0;
    if (method == M_MPFR) {
        if (img->xmin->exp == MDZ_MPFR_EXP_NAN || img->ymax->exp == MDZ_MPFR_EXP_NAN
            || img->width->exp == MDZ_MPFR_EXP_NAN) {
            set_error("view coordinates are NaN");
            return false;
        }
        const mdzgpu_mpval a = as_mpval(img->xmin), b = as_mpval(img->ymax),
                           c = as_mpval(img->width);
        rc = mpfr_coordinate_tables(&a, &b, &c, W, row0, nrows, img->precision, words, xs, ys);
        if (!rc && img->family == MDZ_FAMILY_JULIA) {
            const mdzgpu_mpval jr = as_mpval(img->u.julia.c_re), ji = as_mpval(img->u.julia.c_im);
            rc = mpfr_round_to_fixed(&jr, img->precision, words, jc)
                 | mpfr_round_to_fixed(&ji, img->precision, words, jc + words);
        }
    } else {
        std::vector<uint32_t> a(words), b(words), c(words);
        rc = fx_from_mpf(img->gxmin, words, a.data()) | fx_from_mpf(img->gymax, words, b.data())
             | fx_from_mpf(img->gwidth, words, c.data());
        if (!rc) {
            for (int ix = 0; ix < W; ++ix)
                fx_affine(a.data(), c.data(), ix, W, +1, words, xs + (size_t)ix * words);
            for (int r = 0; r < nrows; ++r)
                fx_affine(b.data(), c.data(), row0 + r, W, -1, words, ys + (size_t)r * words);
            if (img->family == MDZ_FAMILY_JULIA)
                rc = fx_from_mpfr(img->u.julia.c_re, words, jc)
                     | fx_from_mpfr(img->u.julia.c_im, words, jc + words);
        }
    }
    if (rc) {
        set_error("multi-limb path: view outside the fixed-point range (|x|, |y| < 4)");
        return false;
    }
    for (size_t k = 0; k < (size_t)(W + nrows + 2); ++k)
        if (!fx_fits_coordinate(&tab[k * words], words)) {
            set_error("multi-limb path: coordinates must satisfy |x|, |y| < 4");
            return false;
        }
    return true;
}

// Renders the whole frame with one kernel launch, publishing rows as their
// 4-row bands complete.
int gpu_frame(mdz_rthdata* rth, Method method)
{
    mdz_rth_private* d = rth->data;
    mdz_image_info* img = rth->img;
    const int W = img->real_width, H = img->real_height, aa = img->aa_factor;
    const int UH = img->user_height;
    std::vector<char> row_done(UH, 0);
    if (!d->ctx)
        d->ctx = mdzgpu_create(device_index());
    mdzgpu_ctx* ctx = d->ctx;
    if (!ctx) {
        fail_remaining(rth, row_done);
        return 0;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        set_error("cudaSetDevice failed");
        fail_remaining(rth, row_done);
        return 0;
    }
    const int nbands = (H + 3) / 4;
    const size_t n = (size_t)W * H;
    int rc = ctx->staging.ensure(n * sizeof(int32_t));
    if (!rc)
        rc = ctx->pinned.ensure((size_t)(nbands + 64) * sizeof(int));
    if (!rc)
        rc = ctx->sync.ensure(256 + (size_t)nbands * sizeof(unsigned));
    if (rc) {
        fail_remaining(rth, row_done);
        return 0;
    }
    volatile int* hflags = (volatile int*)ctx->pinned.host;
    volatile int* hstop = hflags + nbands;
    memset((void*)hflags, 0, (size_t)(nbands + 1) * sizeof(int));
    int* dflags = (int*)ctx->pinned.dev;
    int* dstop = dflags + nbands;
    FrameSync* dsync = (FrameSync*)ctx->sync.ptr;
    unsigned* dbands = (unsigned*)((char*)ctx->sync.ptr + 256);
    const int32_t* hstaging = (const int32_t*)ctx->staging.host;
    int32_t* dstaging = (int32_t*)ctx->staging.dev;
    cudaStream_t s = ctx->stream;

    if (cudaMemsetAsync(ctx->sync.ptr, 0, 256 + (size_t)nbands * sizeof(unsigned), s) != cudaSuccess) {
        set_error("cudaMemsetAsync failed");
        fail_remaining(rth, row_done);
        return 0;
    }
    if (method == M_FP64) {
        Fp64Launch p;
        p.W = W;
        p.H = H;
        p.row0 = 0;
        p.nrows = H;
        p.family = img->family;
        p.fractal = img->fractal;
        p.depth = (uint32_t)(img->depth > 0x7fffffff ? 0x7fffffff : img->depth);
        // src/fractal.c:50-58: mpfr_get_ld(..., GMP_RNDN), long double = double
        p.xmin = mpfr_to_double_rn(img->xmin);
        p.xmax = mpfr_to_double_rn(img->xmax);
        p.ymax = mpfr_to_double_rn(img->ymax);
        p.jre = img->family == MDZ_FAMILY_JULIA ? mpfr_to_double_rn(img->u.julia.c_re) : 0.0;
        p.jim = img->family == MDZ_FAMILY_JULIA ? mpfr_to_double_rn(img->u.julia.c_im) : 0.0;
        p.out = dstaging;
        p.sync = dsync;
        p.tile_rows_done = dbands;
        p.band_flags = dflags;
        p.stop = dstop;
        rc = launch_fp64(ctx, p, s);
    } else {
        const int words_req = mp_words_for_precision(img->precision);
        int words = -1;
        for (int w = words_req; w <= mdzgpu_mp_max_words(); ++w)
            if (mp_words_supported(w)) {
                words = w;
                break;
            }
        if (words < 0) {
            set_error("precision %ld is beyond the multi-limb kernels", img->precision);
            fail_remaining(rth, row_done);
            return 0;
        }
        std::vector<uint32_t> tab((size_t)(W + H + 2) * words, 0);
        if (!frame_tables(img, method, words, 0, H, tab)) {
            fail_remaining(rth, row_done);
            return 0;
        }
        if ((rc = ctx->coords.ensure(tab.size() * 4))
            || cudaMemcpyAsync(ctx->coords.ptr, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, s)
                   != cudaSuccess
            || cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("coordinate upload failed");
            fail_remaining(rth, row_done);
            return 0;
        }
        MpLaunch p;
        p.W = W;
        p.H = H;
        p.row0 = 0;
        p.nrows = H;
        p.family = img->family;
        p.fractal = img->fractal;
        p.depth = (uint32_t)(img->depth > 0x7fffffff ? 0x7fffffff : img->depth);
        p.words = words;
        p.xs = (const uint32_t*)ctx->coords.ptr;
        p.ys = p.xs + (size_t)W * words;
        p.julia = p.xs + (size_t)(W + H) * words;
        p.out = dstaging;
        p.sync = dsync;
        p.tile_rows_done = dbands;
        p.band_flags = dflags;
        p.stop = dstop;
        rc = launch_mp(ctx, p, s);
    }
    cudaEvent_t done_ev;
    if (rc || cudaEventCreateWithFlags(&done_ev, cudaEventDisableTiming) != cudaSuccess) {
        fail_remaining(rth, row_done);
        return 0;
    }
    cudaEventRecord(done_ev, s);

    // user rows complete when every 4-row band they touch is complete
    std::vector<char> band_seen(nbands, 0);
    int rows_left = UH;
    bool stopping = false;
    bool finished = false;
    while (!finished) {
        if (!stopping && (get_status(d) & (RT_STOP | RT_QUIT))) {
            *hstop = 1;  // kernel warps stop pulling tiles
            stopping = true;
        }
        const cudaError_t q = cudaEventQuery(done_ev);
        if (q != cudaSuccess && q != cudaErrorNotReady) {
            set_error("render kernel failed: %s", cudaGetErrorString(q));
            cudaEventDestroy(done_ev);
            fail_remaining(rth, row_done);
            return 0;
        }
        finished = (q == cudaSuccess);
        bool any = false;
        for (int b = 0; b < nbands; ++b)
            if (!band_seen[b] && hflags[b]) {
                band_seen[b] = 1;
                any = true;
            }
        if (any && !stopping) {
            std::atomic_thread_fence(std::memory_order_acquire);
            for (int y = 0; y < UH; ++y) {
                if (row_done[y])
                    continue;
                const int r0 = y * aa, r1 = y * aa + aa - 1;
                bool ok = true;
                for (int b = r0 / 4; b <= r1 / 4 && ok; ++b)
                    ok = band_seen[b] != 0;
                if (!ok)
                    continue;
                memcpy(img->raw_data + (size_t)r0 * W, hstaging + (size_t)r0 * W,
                       (size_t)aa * W * sizeof(int32_t));
                row_done[y] = 1;
                --rows_left;
                publish_row(rth, y);
            }
        }
        if (!finished)
            usleep(200);
    }
    cudaEventDestroy(done_ev);
    return rows_left == 0 ? 1 : 0;
}

// A callback that is not one of the three line functions: call it row by
// row, as the reference's workers do (src/render_threads.c:360-393).
void host_frame(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    const int aa = rth->img->aa_factor;
    for (int line = 0; line < rth->img->real_height; line += aa) {
        if (get_status(d) & (RT_STOP | RT_QUIT))
            return;
        for (int i = 0; i < aa; ++i)
            if (!d->next_line_cb(rth->img, line + i))
                return;
        publish_row(rth, line / aa);
    }
}

void* render_thread_main(void* arg)
{
    mdz_rthdata* rth = (mdz_rthdata*)arg;
    mdz_rth_private* d = rth->data;
    pthread_mutex_lock(&d->lines_mutex);
    memset(d->lines_rendered, 0, rth->img->user_height);
    d->total_lines_rendered = 0;
    d->min_line_rendered = 0;
    pthread_mutex_unlock(&d->lines_mutex);
    set_status(d, RT_RENDERING);
    if (!rth->check_stop_px)
        rth->check_stop_px = 64;
    rth->thread_count = 1;
    gettimeofday(&d->tv_start, nullptr);
    pthread_mutex_lock(&d->started_mutex);
    d->started = 1;
    pthread_cond_signal(&d->started_cond);
    pthread_mutex_unlock(&d->started_mutex);

    const Method m = classify(d->next_line_cb);
    if (m == M_HOST)
        host_frame(rth);
    else
        gpu_frame(rth, m);

    gettimeofday(&d->tv_end, nullptr);
    set_status(d, RT_STOP);
    return nullptr;
}

void* watch_thread_main(void* arg)
{
    mdz_rthdata* rth = (mdz_rthdata*)arg;
    mdz_rth_private* d = rth->data;
    for (;;) {
        pthread_mutex_lock(&d->start_mutex);
        while (!d->start) {
            // bounded wait so that a quit request signalled under another
            // mutex is never lost (the reference's rth_ui_quit signals
            // start_cond under status_mutex)
            struct timespec ts;
            clock_gettime(CLOCK_REALTIME, &ts);
            ts.tv_nsec += 50 * 1000 * 1000;
            if (ts.tv_nsec >= 1000000000L) {
                ts.tv_sec += 1;
                ts.tv_nsec -= 1000000000L;
            }
            pthread_cond_timedwait(&d->start_cond, &d->start_mutex, &ts);
            if (get_status(d) & RT_QUIT)
                break;
        }
        d->start = 0;
        pthread_mutex_unlock(&d->start_mutex);

        pthread_mutex_lock(&d->started_mutex);
        d->started = 0;
        pthread_mutex_unlock(&d->started_mutex);

        pthread_mutex_lock(&d->status_mutex);
        const int quit = d->status & RT_QUIT;
        const bool rendering = (d->status & RT_RENDERING) != 0;
        if (rendering)
            d->status = RT_STOP | (d->status & RT_QUIT);
        pthread_mutex_unlock(&d->status_mutex);

        if (d->render_live) {
            pthread_join(d->render_thread, nullptr);
            d->render_live = false;
        }
        if (quit)
            return nullptr;
        if (pthread_create(&d->render_thread, nullptr, render_thread_main, rth) != 0) {
            fprintf(stderr, "mdzgpu: failed to create render thread\n");
            return nullptr;
        }
        d->render_live = true;
    }
}

std::mutex g_line_mutex;
mdzgpu_ctx* g_line_ctx = nullptr;

// One real row through the explicit layer (for callers that use the line
// functions directly, as the reference allows).
int line_render(mdz_image_info* img, int line, Method method)
{
    std::lock_guard<std::mutex> lock(g_line_mutex);
    if (!g_line_ctx)
        g_line_ctx = mdzgpu_create(device_index());
    mdzgpu_ctx* ctx = g_line_ctx;
    if (!ctx)
        return 0;
    const int W = img->real_width;
    if (line < 0 || line >= img->real_height)
        return 0;
    int rc = ctx->counts.ensure((size_t)W * sizeof(int32_t));
    if (!rc)
        rc = ctx->sync.ensure(sizeof(FrameSync));
    if (rc)
        return 0;
    cudaSetDevice(ctx->device);
    cudaMemsetAsync(ctx->sync.ptr, 0, sizeof(FrameSync), ctx->stream);
    if (method == M_FP64) {
        Fp64Launch p;
        p.W = W;
        p.H = img->real_height;
        p.row0 = line;
        p.nrows = 1;
        p.family = img->family;
        p.fractal = img->fractal;
        p.depth = (uint32_t)img->depth;
        p.xmin = mpfr_to_double_rn(img->xmin);
        p.xmax = mpfr_to_double_rn(img->xmax);
        p.ymax = mpfr_to_double_rn(img->ymax);
        p.jre = img->family == MDZ_FAMILY_JULIA ? mpfr_to_double_rn(img->u.julia.c_re) : 0.0;
        p.jim = img->family == MDZ_FAMILY_JULIA ? mpfr_to_double_rn(img->u.julia.c_im) : 0.0;
        p.out = (int32_t*)ctx->counts.ptr;
        p.sync = (FrameSync*)ctx->sync.ptr;
        p.tile_rows_done = nullptr;
        p.band_flags = nullptr;
        p.stop = nullptr;
        if (launch_fp64(ctx, p, ctx->stream))
            return 0;
    } else {
        int words = -1;
        for (int w = mp_words_for_precision(img->precision); w <= mdzgpu_mp_max_words(); ++w)
            if (mp_words_supported(w)) {
                words = w;
                break;
            }
        if (words < 0)
            return 0;
        std::vector<uint32_t> tab((size_t)(W + 3) * words, 0);
        if (!frame_tables(img, method, words, line, 1, tab))
            return 0;
        if (ctx->coords.ensure(tab.size() * 4)
            || cudaMemcpyAsync(ctx->coords.ptr, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice,
                               ctx->stream) != cudaSuccess)
            return 0;
        MpLaunch p;
        p.W = W;
        p.H = img->real_height;
        p.row0 = line;
        p.nrows = 1;
        p.family = img->family;
        p.fractal = img->fractal;
        p.depth = (uint32_t)img->depth;
        p.words = words;
        p.xs = (const uint32_t*)ctx->coords.ptr;
        p.ys = p.xs + (size_t)W * words;
        p.julia = p.xs + (size_t)(W + 1) * words;
        p.out = (int32_t*)ctx->counts.ptr;
        p.sync = (FrameSync*)ctx->sync.ptr;
        p.tile_rows_done = nullptr;
        p.band_flags = nullptr;
        p.stop = nullptr;
        if (launch_mp(ctx, p, ctx->stream))
            return 0;
    }
    if (cudaMemcpyAsync(img->raw_data + (size_t)line * W, ctx->counts.ptr, (size_t)W * 4,
                        cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess
        || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        set_error("line render failed");
        return 0;
    }
    if (img->rth_ptr && rth_render_should_stop((mdz_rthdata*)img->rth_ptr))
        return 0;
    return 1;
}

}  // namespace

extern "C" {

mdz_rthdata* rth_create(void)
{
    mdz_rthdata* rth = (mdz_rthdata*)calloc(1, sizeof(mdz_rthdata));
    if (!rth)
        return nullptr;
    rth->data = new (std::nothrow) mdz_rth_private();
    if (!rth->data) {
        free(rth);
        return nullptr;
    }
    return rth;
}

int rth_init(mdz_rthdata* rth, int thread_count, int line_draw_count, mdz_image_info* img)
{
    if (img)
        rth->img = img;
    mdz_rth_private* d = rth->data;
    if (thread_count)
        d->thread_count = thread_count;
    d->start = 0;
    d->status = 0;
    free(d->lines_rendered);
    free(rth->lines_drawn);
    d->lines_rendered = (char*)calloc((size_t)rth->img->user_height, 1);
    rth->lines_drawn = (char*)calloc((size_t)rth->img->user_height, 1);
    if (!d->lines_rendered || !rth->lines_drawn)
        return 0;
    d->min_line_rendered = 0;
    rth->min_line_drawn = 0;
    rth->line_draw_count = line_draw_count;
    if (!d->initialized) {
        d->initialized = true;
        pthread_mutex_init(&d->start_mutex, nullptr);
        pthread_mutex_init(&d->started_mutex, nullptr);
        pthread_mutex_init(&d->status_mutex, nullptr);
        pthread_mutex_init(&d->lines_mutex, nullptr);
        pthread_cond_init(&d->start_cond, nullptr);
        pthread_cond_init(&d->started_cond, nullptr);
        pthread_cond_init(&d->lines_cond, nullptr);
    }
    return 1;
}

int rth_ui_init(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    if (pthread_create(&d->watch_thread, nullptr, watch_thread_main, rth) != 0) {
        fprintf(stderr, "Failed to create start_watch thread\n");
        return 0;
    }
    d->watch_live = true;
    return 1;
}

void rth_ui_start_render(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    memset(rth->lines_drawn, 0, (size_t)rth->img->user_height);
    rth->min_line_drawn = 0;
    // Reset the progress of the previous frame here, not only when the new
    // render thread starts: a caller that waits for lines straight after
    // this call (render.c:49-51) must not see the last frame as finished.
    pthread_mutex_lock(&d->lines_mutex);
    memset(d->lines_rendered, 0, (size_t)rth->img->user_height);
    d->total_lines_rendered = 0;
    d->min_line_rendered = 0;
    pthread_mutex_unlock(&d->lines_mutex);
    pthread_mutex_lock(&d->started_mutex);
    d->started = 0;
    pthread_mutex_unlock(&d->started_mutex);
    pthread_mutex_lock(&d->start_mutex);
    d->start = 1;
    pthread_cond_signal(&d->start_cond);
    pthread_mutex_unlock(&d->start_mutex);
}

void rth_ui_stop_render(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    pthread_mutex_lock(&d->status_mutex);
    d->status = RT_STOP | (d->status & RT_RENDERING);
    pthread_mutex_unlock(&d->status_mutex);
}

void rth_ui_stop_render_and_wait(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    pthread_mutex_lock(&d->status_mutex);
    if (d->status & RT_STOP) {
        pthread_mutex_unlock(&d->status_mutex);
        return;
    }
    d->status = RT_STOP | (d->status & RT_RENDERING);
    pthread_mutex_unlock(&d->status_mutex);
    // wait until the render thread has left the GPU loop
    while (get_status(d) & RT_RENDERING)
        usleep(200);
}

void rth_ui_quit(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    pthread_mutex_lock(&d->status_mutex);
    d->status |= RT_QUIT;
    pthread_mutex_unlock(&d->status_mutex);
    pthread_mutex_lock(&d->start_mutex);
    pthread_cond_signal(&d->start_cond);
    pthread_mutex_unlock(&d->start_mutex);
    if (d->watch_live) {
        pthread_join(d->watch_thread, nullptr);
        d->watch_live = false;
    }
    if (d->render_live) {
        pthread_join(d->render_thread, nullptr);
        d->render_live = false;
    }
    if (d->ctx) {
        mdzgpu_destroy(d->ctx);
        d->ctx = nullptr;
    }
    free(d->lines_rendered);
    free(rth->lines_drawn);
    d->lines_rendered = nullptr;
    rth->lines_drawn = nullptr;
}

void rth_ui_wait_until_started(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    pthread_mutex_lock(&d->started_mutex);
    while (!d->started)
        pthread_cond_wait(&d->started_cond, &d->started_mutex);
    pthread_cond_signal(&d->started_cond);
    pthread_mutex_unlock(&d->started_mutex);
}

void rth_set_next_line_cb(mdz_rthdata* rth, int (*next_line_cb)(mdz_image_info*, int))
{
    rth->data->next_line_cb = next_line_cb;
}

int rth_process_lines_rendered(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    const int height = rth->img->user_height;
    pthread_mutex_lock(&d->lines_mutex);
    const int linesdone = d->total_lines_rendered / rth->img->aa_factor;
    const int miny = d->min_line_rendered;
    pthread_mutex_unlock(&d->lines_mutex);
    if (miny == linesdone)
        return 0;
    int maxy = miny + rth->line_draw_count + 1;
    if (maxy > height)
        maxy = height;
    if (maxy > linesdone)
        maxy = linesdone;
    if (miny < maxy) {
        pthread_mutex_lock(&d->lines_mutex);
        int unrendered = 0;
        for (int i = miny; i < maxy; ++i) {
            if (d->lines_rendered[i] == 1) {
                d->lines_rendered[i] = 2;
                rth->lines_drawn[i] = 1;
                if (!unrendered)
                    d->min_line_rendered = i;
            } else if (d->lines_rendered[i] == 0) {
                unrendered = 1;
            }
        }
        pthread_mutex_unlock(&d->lines_mutex);
    }
    return (linesdone < height) ? linesdone : -1;
}

int rth_render_should_stop(mdz_rthdata* rth)
{
    return (get_status(rth->data) & RT_STOP) ? 1 : 0;
}

int rth_ui_wait_for_line_done(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    pthread_mutex_lock(&d->lines_mutex);
    if (d->total_lines_rendered == rth->img->real_height) {
        pthread_mutex_unlock(&d->lines_mutex);
        return -1;
    }
    struct timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    ts.tv_nsec += 100 * 1000 * 1000;
    if (ts.tv_nsec >= 1000000000L) {
        ts.tv_sec += 1;
        ts.tv_nsec -= 1000000000L;
    }
    pthread_cond_timedwait(&d->lines_cond, &d->lines_mutex, &ts);
    const int linesdone = d->total_lines_rendered / rth->img->aa_factor;
    pthread_mutex_unlock(&d->lines_mutex);
    return (linesdone < rth->img->user_height) ? linesdone : -1;
}

void rth_ui_stop_timer(mdz_rthdata* rth)
{
    gettimeofday(&rth->data->tv_end, nullptr);
}

double rth_ui_get_render_time(mdz_rthdata* rth)
{
    mdz_rth_private* d = rth->data;
    if (get_status(d) & RT_RENDERING)
        gettimeofday(&d->tv_end, nullptr);
    return (d->tv_end.tv_sec - d->tv_start.tv_sec) + (d->tv_end.tv_usec - d->tv_start.tv_usec) * 1e-6;
}

int fractal_calculate_line(mdz_image_info* img, int line)
{
    return line_render(img, line, M_FP64);
}

int fractal_mpfr_calculate_line(mdz_image_info* img, int line)
{
    return line_render(img, line, M_MPFR);
}

int fractal_gmp_calculate_line(mdz_image_info* img, int line)
{
    return line_render(img, line, M_GMP);
}

}  // extern "C"
