/* CPU oracle for the MDZ escape-time hot path -- TEST INFRASTRUCTURE.
 *
 * A plain-C restatement of the reference's algorithm, used only by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker and
 * the CPU baseline.  Never linked into libmdzgpu.
 *
 *   mdzo_render_fp64   fractal_calculate_line (src/fractal.c:29-117) with
 *                      long double = IEEE double, no FMA (built with
 *                      -ffp-contract=off), driven by a row pool that
 *                      restates rth_next_line (src/render_threads.c:360-393):
 *                      a mutex-protected next_line counter advanced by aa.
 *   frac loops         src/frac_mandel.c:5-21, src/frac_burning_ship.c:7-24,
 *                      src/frac_generalized_celtic.c:7-24,
 *                      src/frac_variant.c:5-24.
 *   mdzo_render_mpfr   fractal_mpfr_calculate_line (src/fractal.c:120-257)
 *                      and the frac_*_mpfr loops (src/frac_mandel.c:25-52
 *                      etc.) calling the system MPFR with round-to-nearest;
 *                      compiled only when libmpfr.so.6 is found
 *                      (MDZO_WITH_MPFR).
 *   mdzo_points_mpfr   the same per-pixel MPFR loop on an explicit list of
 *                      c values, also returning |z|^2 at escape (the
 *                      reference returns the count only), for the
 *                      perturbation and smooth-colour scoring.
 * Thread counts are explicit so the CPU baseline states the cores it used. */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---- colouring (TEST INFRASTRUCTURE restatement) ----
 * palette_apply (src/palette.c:406-463) for aa = 1 and do_anti_aliasing
 * (src/render.c:108-158) through get_pixel_colour (src/palette.c:466-503)
 * for aa > 1, on raw counts `raw` [real_h][real_w] into rgb [user_h][user_w].
 * Colours use MDZ's little-endian packing r | g << 8 | b << 16.  Doubles are
 * formed exactly as the C code forms them (this file is built without FMA
 * contraction).  Defined for 0 <= raw * scale + offset < 2^31. */
#define MDZO_RED(x) ((x) & 0xffu)
#define MDZO_GREEN(x) (((x) & 0xff00u) >> 8)
#define MDZO_BLUE(x) (((x) & 0xff0000u) >> 16)
#define MDZO_RGB(r, g, b) ((uint32_t)(r) | ((uint32_t)(g) << 8) | ((uint32_t)(b) << 16))

static uint32_t colour_of(double val, int ip, const uint32_t* pal, int n, int off)
{
    if (val)
        val += off;
    if (ip) {
        const double cval = ceil(val);
        const double diff = cval - val;
        const double rdiff = 1.0 - diff;
        const uint32_t i1 = ((uint32_t)floor(val)) % (uint32_t)(n - 1);
        const uint32_t i2 = (uint32_t)cval % (uint32_t)(n - 1);
        const uint32_t c1 = pal[i1], c2 = pal[i2];
        const uint8_t r = (uint8_t)(diff * MDZO_RED(c1) + rdiff * MDZO_RED(c2));
        const uint8_t g = (uint8_t)(diff * MDZO_GREEN(c1) + rdiff * MDZO_GREEN(c2));
        const uint8_t b = (uint8_t)(diff * MDZO_BLUE(c1) + rdiff * MDZO_BLUE(c2));
        return MDZO_RGB(r, g, b);
    }
    if (val == 0)
        return 0;
    return pal[(uint32_t)val % (uint32_t)(n - 1)];
}

int mdzo_colour(const int32_t* raw, int real_w, int real_h, int aa, int ip, double sc,
                const uint32_t* pal, int n, int off, uint32_t* rgb)
{
    if (aa < 1 || real_w % aa || real_h % aa || n < 2 || n > 256)
        return 0;
    const int uw = real_w / aa, uh = real_h / aa;
    for (int y = 0; y < uh; ++y) {
        for (int x = 0; x < uw; ++x) {
            if (aa == 1) {
                const int v = raw[(size_t)y * real_w + x];
                uint32_t out = 0;
                if (v) {
                    const double ip_val = v * sc + off;
                    if (ip) {
                        const int ip_cval = (int)ceil(ip_val);
                        const double ip_diff = ip_cval - ip_val;
                        const double ip_rdiff = 1.0 - ip_diff;
                        const int i1 = (int)floor(ip_val) % (n - 1);
                        const int i2 = ip_cval % (n - 1);
                        const uint32_t c1 = pal[i1], c2 = pal[i2];
                        const uint8_t r = (uint8_t)(ip_diff * MDZO_RED(c1) + ip_rdiff * MDZO_RED(c2));
                        const uint8_t g =
                            (uint8_t)(ip_diff * MDZO_GREEN(c1) + ip_rdiff * MDZO_GREEN(c2));
                        const uint8_t b =
                            (uint8_t)(ip_diff * MDZO_BLUE(c1) + ip_rdiff * MDZO_BLUE(c2));
                        out = MDZO_RGB(r, g, b);
                    } else {
                        out = pal[(uint32_t)ip_val % (uint32_t)(n - 1)];
                    }
                }
                rgb[(size_t)y * uw + x] = out;
            } else {
                uint32_t r = 0, g = 0, b = 0;
                for (int yi = y * aa; yi < y * aa + aa; ++yi)
                    for (int xi = x * aa; xi < x * aa + aa; ++xi) {
                        const uint32_t c =
                            colour_of(raw[(size_t)yi * real_w + xi] * sc, ip, pal, n, off);
                        r += MDZO_RED(c);
                        g += MDZO_GREEN(c);
                        b += MDZO_BLUE(c);
                    }
                const uint32_t a2 = (uint32_t)(aa * aa);
                rgb[(size_t)y * uw + x] = MDZO_RGB(r / a2, g / a2, b / a2);
            }
        }
    }
    return 1;
}

#ifdef MDZO_WITH_MPFR
#include "mpfr.h"
#endif

enum { MANDELBROT = 0, BURNING_SHIP = 1, GENERALIZED_CELTIC = 2, VARIANT = 3 };
enum { FAMILY_MANDEL = 0, FAMILY_JULIA = 1 };

/* ---- hardware-float loops (double) ---- */

static int64_t frac_fp64(int fractal, int64_t depth, double wim, double wre,
                         double c_im, double c_re, double wim2, double wre2)
{
    int64_t wz;
    for (wz = 1; wz <= depth; ++wz) {
        if (fractal == BURNING_SHIP)
            wim = 2.0 * fabs(wre * wim) + c_im;
        else
            wim = 2.0 * wre * wim + c_im;
        if (fractal == GENERALIZED_CELTIC || (fractal == VARIANT && (wz % 2)))
            wre = fabs(wre2 - wim2) + c_re;
        else
            wre = wre2 - wim2 + c_re;
        wim2 = wim * wim;
        wre2 = wre * wre;
        if (wim2 + wre2 > 4.0F)
            return wz;
    }
    return 0;
}

typedef struct {
    int W, H, aa, family, fractal, nthreads;
    int64_t depth;
    double xmin, xmax, ymax, jre, jim;
    int32_t* out;
    int next_line;
    int64_t pixel_iters;
    pthread_mutex_t mu;
#ifdef MDZO_WITH_MPFR
    long prec;
    const char *s_xmin, *s_ymax, *s_width, *s_jre, *s_jim;
    long p_xmin, p_ymax, p_width, p_jre, p_jim;
#endif
} frame_job;

static void fp64_line(frame_job* j, int line)
{
    const double width = j->xmax - j->xmin;
    const double y = j->ymax - (width / (double)j->W) * (double)line;
    const double y2 = y * y;
    int32_t* raw = j->out + (size_t)line * j->W;
    int64_t its = 0;
    for (int ix = 0; ix < j->W; ++ix) {
        const double x = (ix / (double)j->W) * width + j->xmin;
        const double x2 = x * x;
        double c_re = x, c_im = y;
        if (j->family == FAMILY_JULIA) {
            c_re = j->jre;
            c_im = j->jim;
        }
        const int64_t n = frac_fp64(j->fractal, j->depth, y, x, c_im, c_re, y2, x2);
        raw[ix] = (int32_t)n;
        its += n ? n : j->depth;
    }
    pthread_mutex_lock(&j->mu);
    j->pixel_iters += its;
    pthread_mutex_unlock(&j->mu);
}

/* rth_next_line: grab aa rows at a time under the mutex */
static int grab(frame_job* j)
{
    pthread_mutex_lock(&j->mu);
    const int line = j->next_line;
    j->next_line += j->aa;
    pthread_mutex_unlock(&j->mu);
    return line < j->H ? line : -1;
}

static void* fp64_worker(void* arg)
{
    frame_job* j = (frame_job*)arg;
    int line;
    while ((line = grab(j)) >= 0)
        for (int i = 0; i < j->aa && line + i < j->H; ++i)
            fp64_line(j, line + i);
    return 0;
}

static int run_pool(frame_job* j, void* (*fn)(void*))
{
    int n = j->nthreads < 1 ? 1 : j->nthreads;
    pthread_t* th = (pthread_t*)calloc((size_t)n, sizeof(pthread_t));
    if (!th)
        return -1;
    for (int i = 0; i < n; ++i)
        if (pthread_create(&th[i], 0, fn, j)) {
            n = i;
            break;
        }
    for (int i = 0; i < n; ++i)
        pthread_join(th[i], 0);
    free(th);
    return 0;
}

/* Renders rows [0, H) of a W x H frame; returns the pixel-iteration sum. */
int64_t mdzo_render_fp64(int W, int H, int aa, int64_t depth, int family, int fractal,
                         double xmin, double xmax, double ymax, double jre, double jim,
                         int nthreads, int32_t* out)
{
    frame_job j;
    memset(&j, 0, sizeof j);
    j.W = W;
    j.H = H;
    j.aa = aa < 1 ? 1 : aa;
    j.depth = depth;
    j.family = family;
    j.fractal = fractal;
    j.xmin = xmin;
    j.xmax = xmax;
    j.ymax = ymax;
    j.jre = jre;
    j.jim = jim;
    j.out = out;
    j.nthreads = nthreads;
    pthread_mutex_init(&j.mu, 0);
    run_pool(&j, fp64_worker);
    pthread_mutex_destroy(&j.mu);
    return j.pixel_iters;
}

/* Rows [row0, row0 + nrows) of a W x H frame into out (nrows x W). */
int64_t mdzo_render_fp64_rows(int W, int H, int row0, int nrows, int64_t depth, int family,
                              int fractal, double xmin, double xmax, double ymax, double jre,
                              double jim, int nthreads, int32_t* out)
{
    frame_job j;
    memset(&j, 0, sizeof j);
    j.W = W;
    j.H = row0 + nrows;
    j.aa = 1;
    j.next_line = row0;
    j.depth = depth;
    j.family = family;
    j.fractal = fractal;
    j.xmin = xmin;
    j.xmax = xmax;
    j.ymax = ymax;
    j.jre = jre;
    j.jim = jim;
    j.out = out - (size_t)row0 * W;
    j.nthreads = nthreads;
    (void)H;
    pthread_mutex_init(&j.mu, 0);
    run_pool(&j, fp64_worker);
    pthread_mutex_destroy(&j.mu);
    return j.pixel_iters;
}

/* One Mandelbrot-family pixel through the double loop (z0 = c). */
int64_t mdzo_point_fp64(int fractal, int64_t depth, double c_re, double c_im)
{
    return frac_fp64(fractal, depth, c_im, c_re, c_im, c_re, c_im * c_im, c_re * c_re);
}

#ifdef MDZO_WITH_MPFR

/* frac_*_mpfr, one loop for the four formulas; *mag2 gets |z|^2 (the value
 * compared with the bailout) at the returned iteration. */
static int64_t frac_mpfr(int fractal, int64_t depth, mpfr_t bail, mpfr_t wim, mpfr_t wre,
                         mpfr_t c_im, mpfr_t c_re, mpfr_t wim2, mpfr_t wre2, mpfr_t t1,
                         double* mag2)
{
    int64_t wz;
    for (wz = 1; wz <= depth; wz++) {
        mpfr_mul(t1, wre, wim, GMP_RNDN);
        if (fractal == BURNING_SHIP)
            mpfr_abs(t1, t1, GMP_RNDN);
        mpfr_mul_si(t1, t1, 2, GMP_RNDN);
        mpfr_add(wim, t1, c_im, GMP_RNDN);
        mpfr_sub(t1, wre2, wim2, GMP_RNDN);
        if (fractal == GENERALIZED_CELTIC || (fractal == VARIANT && (wz % 2)))
            mpfr_abs(t1, t1, GMP_RNDN);
        mpfr_add(wre, t1, c_re, GMP_RNDN);
        mpfr_mul(wim2, wim, wim, GMP_RNDN);
        mpfr_mul(wre2, wre, wre, GMP_RNDN);
        mpfr_add(t1, wim2, wre2, GMP_RNDN);
        if (mpfr_greater_p(t1, bail)) {
            if (mag2)
                *mag2 = mpfr_get_d(t1, GMP_RNDN);
            return wz;
        }
    }
    if (mag2)
        *mag2 = mpfr_get_d(t1, GMP_RNDN);
    return 0;
}

typedef struct {
    mpfr_t x, y, x2, y2, c_re, c_im, wre, wim, wre2, wim2, bail, width, img_rw, img_xmin, t1;
    mpfr_t ymax, jre, jim;
} mp_vars;

static void mp_vars_init(mp_vars* v, frame_job* j)
{
    mpfr_t* all[] = {&v->x, &v->y, &v->x2, &v->y2, &v->c_re, &v->c_im, &v->wre, &v->wim,
                     &v->wre2, &v->wim2, &v->bail, &v->width, &v->img_rw, &v->img_xmin, &v->t1};
    for (size_t i = 0; i < sizeof all / sizeof all[0]; ++i)
        mpfr_init2(*all[i], j->prec);
    /* the view values at their own precisions, as image_info holds them */
    mpfr_init2(v->ymax, j->p_ymax);
    mpfr_init2(v->jre, j->p_jre);
    mpfr_init2(v->jim, j->p_jim);
    mpfr_t xmin, width;
    mpfr_init2(xmin, j->p_xmin);
    mpfr_init2(width, j->p_width);
    mpfr_set_str(xmin, j->s_xmin, 0, GMP_RNDN);
    mpfr_set_str(width, j->s_width, 0, GMP_RNDN);
    mpfr_set_str(v->ymax, j->s_ymax, 0, GMP_RNDN);
    mpfr_set_str(v->jre, j->s_jre, 0, GMP_RNDN);
    mpfr_set_str(v->jim, j->s_jim, 0, GMP_RNDN);
    mpfr_set_si(v->bail, 4, GMP_RNDN);
    mpfr_set_si(v->img_rw, j->W, GMP_RNDN);
    mpfr_set(v->img_xmin, xmin, GMP_RNDN);
    mpfr_set(v->width, width, GMP_RNDN);
    mpfr_clear(xmin);
    mpfr_clear(width);
}

static void mp_vars_clear(mp_vars* v)
{
    mpfr_t* all[] = {&v->x, &v->y, &v->x2, &v->y2, &v->c_re, &v->c_im, &v->wre, &v->wim,
                     &v->wre2, &v->wim2, &v->bail, &v->width, &v->img_rw, &v->img_xmin, &v->t1,
                     &v->ymax, &v->jre, &v->jim};
    for (size_t i = 0; i < sizeof all / sizeof all[0]; ++i)
        mpfr_clear(*all[i]);
}

static void mpfr_line(frame_job* j, mp_vars* v, int line)
{
    int32_t* raw = j->out + (size_t)line * j->W;
    int64_t its = 0;
    mpfr_div(v->t1, v->width, v->img_rw, GMP_RNDN);
    mpfr_mul_si(v->t1, v->t1, line, GMP_RNDN);
    mpfr_sub(v->y, v->ymax, v->t1, GMP_RNDN);
    mpfr_mul(v->y2, v->y, v->y, GMP_RNDN);
    for (int ix = 0; ix < j->W; ++ix) {
        mpfr_si_div(v->t1, ix, v->img_rw, GMP_RNDN);
        mpfr_mul(v->x, v->t1, v->width, GMP_RNDN);
        mpfr_add(v->x, v->x, v->img_xmin, GMP_RNDN);
        mpfr_mul(v->x2, v->x, v->x, GMP_RNDN);
        mpfr_set(v->wre, v->x, GMP_RNDN);
        mpfr_set(v->wim, v->y, GMP_RNDN);
        mpfr_set(v->wre2, v->x2, GMP_RNDN);
        mpfr_set(v->wim2, v->y2, GMP_RNDN);
        if (j->family == FAMILY_JULIA) {
            mpfr_set(v->c_re, v->jre, GMP_RNDN);
            mpfr_set(v->c_im, v->jim, GMP_RNDN);
        } else {
            mpfr_set(v->c_re, v->x, GMP_RNDN);
            mpfr_set(v->c_im, v->y, GMP_RNDN);
        }
        const int64_t n = frac_mpfr(j->fractal, j->depth, v->bail, v->wim, v->wre, v->c_im,
                                    v->c_re, v->wim2, v->wre2, v->t1, 0);
        raw[ix] = (int32_t)n;
        its += n ? n : j->depth;
    }
    pthread_mutex_lock(&j->mu);
    j->pixel_iters += its;
    pthread_mutex_unlock(&j->mu);
}

static void* mpfr_worker(void* arg)
{
    frame_job* j = (frame_job*)arg;
    mp_vars v;
    mp_vars_init(&v, j);
    int line;
    while ((line = grab(j)) >= 0)
        for (int i = 0; i < j->aa && line + i < j->H; ++i)
            mpfr_line(j, &v, line + i);
    mp_vars_clear(&v);
    mpfr_free_cache();
    return 0;
}

/* Multiprecision frame (MPFR path).  View values are strings accepted by
 * mpfr_set_str with base 0 (e.g. "-0x1.8p-3"), each parsed at the precision
 * image_info holds it with (p_*). Rows [row0, row0+nrows) of the frame are
 * rendered into out (nrows x W). Returns the pixel-iteration sum. */
int64_t mdzo_render_mpfr(int W, int H, int row0, int nrows, int64_t depth, int family,
                         int fractal, long prec, const char* xmin, long p_xmin,
                         const char* ymax, long p_ymax, const char* width, long p_width,
                         const char* jre, long p_jre, const char* jim, long p_jim,
                         int nthreads, int32_t* out)
{
    frame_job j;
    memset(&j, 0, sizeof j);
    j.W = W;
    j.H = row0 + nrows;
    j.aa = 1;
    j.next_line = row0;
    j.depth = depth;
    j.family = family;
    j.fractal = fractal;
    j.prec = prec;
    j.s_xmin = xmin;
    j.s_ymax = ymax;
    j.s_width = width;
    j.s_jre = jre;
    j.s_jim = jim;
    j.p_xmin = p_xmin;
    j.p_ymax = p_ymax;
    j.p_width = p_width;
    j.p_jre = p_jre;
    j.p_jim = p_jim;
    j.out = out - (size_t)row0 * W;
    j.nthreads = nthreads;
    pthread_mutex_init(&j.mu, 0);
    run_pool(&j, mpfr_worker);
    pthread_mutex_destroy(&j.mu);
    return j.pixel_iters;
}

typedef struct {
    int n, fractal;
    int64_t depth;
    long prec;
    const char* const* cre;
    const char* const* cim;
    const char* jre;  /* Julia family: fixed c (z0 = the listed point) */
    const char* jim;
    int64_t* counts;
    double* mag2;
    int next;
    pthread_mutex_t mu;
} points_job;

static void* points_worker(void* arg)
{
    points_job* j = (points_job*)arg;
    mpfr_t bail, wim, wre, c_im, c_re, wim2, wre2, t1;
    mpfr_init2(bail, j->prec);
    mpfr_init2(wim, j->prec);
    mpfr_init2(wre, j->prec);
    mpfr_init2(c_im, j->prec);
    mpfr_init2(c_re, j->prec);
    mpfr_init2(wim2, j->prec);
    mpfr_init2(wre2, j->prec);
    mpfr_init2(t1, j->prec);
    mpfr_set_si(bail, 4, GMP_RNDN);
    for (;;) {
        pthread_mutex_lock(&j->mu);
        const int i = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (i >= j->n)
            break;
        mpfr_set_str(wre, j->cre[i], 0, GMP_RNDN);
        mpfr_set_str(wim, j->cim[i], 0, GMP_RNDN);
        if (j->jre) {
            mpfr_set_str(c_re, j->jre, 0, GMP_RNDN);
            mpfr_set_str(c_im, j->jim, 0, GMP_RNDN);
        } else {
            mpfr_set(c_re, wre, GMP_RNDN);
            mpfr_set(c_im, wim, GMP_RNDN);
        }
        mpfr_mul(wre2, wre, wre, GMP_RNDN);
        mpfr_mul(wim2, wim, wim, GMP_RNDN);
        double m2 = 0.0;
        j->counts[i] = frac_mpfr(j->fractal, j->depth, bail, wim, wre, c_im, c_re, wim2, wre2, t1,
                                 &m2);
        if (j->mag2)
            j->mag2[i] = m2;
    }
    mpfr_clear(bail);
    mpfr_clear(wim);
    mpfr_clear(wre);
    mpfr_clear(c_im);
    mpfr_clear(c_re);
    mpfr_clear(wim2);
    mpfr_clear(wre2);
    mpfr_clear(t1);
    mpfr_free_cache();
    return 0;
}

/* n Mandelbrot-family pixels c_i (strings, parsed at `prec` bits) through the
 * MPFR loop; counts[i] and |z|^2 at escape (mag2, nullable). */
int mdzo_points_julia_mpfr(int n, int fractal, int64_t depth, long prec,
                           const char* const* zre, const char* const* zim, const char* jre,
                           const char* jim, int nthreads, int64_t* counts, double* mag2);

int mdzo_points_mpfr(int n, int fractal, int64_t depth, long prec, const char* const* cre,
                     const char* const* cim, int nthreads, int64_t* counts, double* mag2)
{
    return mdzo_points_julia_mpfr(n, fractal, depth, prec, cre, cim, 0, 0, nthreads, counts,
                                  mag2);
}

/* Julia family (jre != NULL): z0 = the listed points, c = (jre, jim). */
int mdzo_points_julia_mpfr(int n, int fractal, int64_t depth, long prec,
                           const char* const* cre, const char* const* cim, const char* jre,
                           const char* jim, int nthreads, int64_t* counts, double* mag2)
{
    points_job j;
    memset(&j, 0, sizeof j);
    j.jre = jre;
    j.jim = jim;
    j.n = n;
    j.fractal = fractal;
    j.depth = depth;
    j.prec = prec;
    j.cre = cre;
    j.cim = cim;
    j.counts = counts;
    j.mag2 = mag2;
    pthread_mutex_init(&j.mu, 0);
    int nt = nthreads < 1 ? 1 : nthreads;
    pthread_t* th = (pthread_t*)calloc((size_t)nt, sizeof(pthread_t));
    for (int i = 0; i < nt; ++i)
        pthread_create(&th[i], 0, points_worker, &j);
    for (int i = 0; i < nt; ++i)
        pthread_join(th[i], 0);
    free(th);
    pthread_mutex_destroy(&j.mu);
    return 0;
}

int mdzo_has_mpfr(void)
{
    return 1;
}

#else

int mdzo_has_mpfr(void)
{
    return 0;
}

#endif
