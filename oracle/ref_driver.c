/* Driver for the UNMODIFIED MDZ hot path (TEST INFRASTRUCTURE, oracle).
 *
 * Compiled by oracle/build_ref.sh together with MDZ's own
 *   src/frac_mandel.c src/frac_burning_ship.c src/frac_generalized_celtic.c
 *   src/frac_variant.c src/fractal.c src/render_threads.c src/coords.c
 *   src/my_mpfr_to_str.c src/timer.c src/debug.c
 * into oracle/_ref/libmdzref_{d,ld}.so.  Nothing in the product links it.
 *
 * It sets up an image_info the way MDZ's headless `--render` path does and
 * renders through the reference's own rth_* thread pool:
 *   image_info_create           src/image_info.c:29-76
 *   image_info_load_settings    src/image_info.c:456-721 (centre/size form)
 *   image_info_set              src/image_info.c:104-144
 *   image_info_set_precision    src/image_info.c:252-280
 *   image_info_set_multi_prec   src/image_info.c:226-249
 *   render_to_file              src/render.c:24-94
 * image_info.c itself is not compiled (it pulls in GTK, libpng and the
 * palette code), so those few steps are restated below; every arithmetic
 * step on the coordinates and every pixel is MDZ's own code (coords.c,
 * fractal.c, frac_*.c) linked against the system MPFR/GMP. */
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <unistd.h>

#include "image_info.h"
#include "render_threads.h"
#include "fractal.h"
#include "coords.h"
#include "cmdline.h"
#include "frac_mandel.h"
#include "frac_burning_ship.h"
#include "frac_generalized_celtic.h"
#include "frac_variant.h"

options opts; /* referenced by cmdline.h users; unused on this path */

static double now_s(void)
{
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + tv.tv_usec * 1e-6;
}

/* image_info_set_precision (src/image_info.c:252-280), including its
 * behaviour of changing u.julia.c_re twice and leaving c_im at 80 bits. */
static void set_precision(image_info* img, mpfr_prec_t precision)
{
    if (img->precision == precision)
        return;
    img->precision = precision;
    if (precision < DEFAULT_PRECISION)
        precision = DEFAULT_PRECISION;
    precision_change(img->xmin, precision);
    precision_change(img->xmax, precision);
    precision_change(img->ymax, precision);
    precision_change(img->width, precision);
    precision_change(img->old_cx, precision);
    precision_change(img->old_cy, precision);
    precision_change(img->old_size, precision);
    precision_change(img->u.julia.c_re, precision);
    precision_change(img->u.julia.c_re, precision);
    precision_change_gmp(img->gxmin, precision);
    precision_change_gmp(img->gxmax, precision);
    precision_change_gmp(img->gymax, precision);
    precision_change_gmp(img->gwidth, precision);
    coords_set_precision(img->pcoords, precision);
}

static void set_multi_prec(image_info* img, int mp, int rounding)
{
    rthdata* rth = (rthdata*)img->rth_ptr;
    img->use_multi_prec = mp;
    if (mp) {
        img->use_rounding = rounding;
        rth_set_next_line_cb(rth, rounding ? fractal_mpfr_calculate_line
                                           : fractal_gmp_calculate_line);
    } else {
        rth_set_next_line_cb(rth, fractal_calculate_line);
    }
}

/* image_info_set (src/image_info.c:104-144) minus the RGB buffer. */
static int set_size(image_info* img, int w, int h, int aa)
{
    free(img->raw_data);
    img->user_width = w;
    img->user_height = h;
    img->aa_factor = (aa < 1) ? 1 : aa;
    img->aspect = (double)w / h;
    coords_set(img->pcoords, img->user_width, img->user_height);
    img->real_width = w * aa;
    img->real_height = h * aa;
    img->raw_data = malloc((size_t)img->real_width * img->real_height * sizeof(int));
    if (!img->raw_data)
        return 0;
    for (long i = 0; i < (long)img->real_width * img->real_height; i++)
        img->raw_data[i] = UINT_MAX;
    if (!img->rth_ptr) {
        img->rth_ptr = rth_create();
        if (!img->rth_ptr)
            return 0;
    }
    if (!rth_init((rthdata*)img->rth_ptr, img->thread_count, img->draw_lines, img))
        return 0;
    set_multi_prec(img, img->use_multi_prec, img->use_rounding);
    return 1;
}

static image_info* build_view(int w, int h, int aa, long depth, int family,
                              int fractal, int multi_prec, int rounding,
                              long precision, const char* cx, const char* cy,
                              const char* size, const char* jre,
                              const char* jim, int threads)
{
    image_info* img = calloc(1, sizeof(*img));
    if (!img)
        return 0;
    /* image_info_create */
    img->family = family;
    img->fractal = fractal;
    img->real_width = img->user_width = DEFAULT_WIDTH;
    img->real_height = img->user_height = DEFAULT_HEIGHT;
    img->aspect = DEFAULT_ASPECT;
    img->draw_lines = 64;
    img->thread_count = threads;
    mpfr_init2(img->xmin, DEFAULT_PRECISION);
    mpfr_init2(img->xmax, DEFAULT_PRECISION);
    mpfr_init2(img->ymax, DEFAULT_PRECISION);
    mpfr_init2(img->width, DEFAULT_PRECISION);
    mpfr_init2(img->old_cx, DEFAULT_PRECISION);
    mpfr_init2(img->old_cy, DEFAULT_PRECISION);
    mpfr_init2(img->old_size, DEFAULT_PRECISION);
    mpfr_init2(img->u.julia.c_re, DEFAULT_PRECISION);
    mpfr_init2(img->u.julia.c_im, DEFAULT_PRECISION);
    mpf_init2(img->gxmin, DEFAULT_PRECISION);
    mpf_init2(img->gxmax, DEFAULT_PRECISION);
    mpf_init2(img->gymax, DEFAULT_PRECISION);
    mpf_init2(img->gwidth, DEFAULT_PRECISION);
    img->pcoords = coords_new(img->real_width, img->real_height,
                              family == FAMILY_JULIA ? 0.0 : -0.5, 0.0, 4.0);
    /* image_info_reset_view */
    img->depth = 300;
    img->precision = DEFAULT_PRECISION;
    coords_reset(img->pcoords);

    /* image_info_load_settings, centre/size form */
    mpfr_t m_cx, m_cy, m_size, m_jre, m_jim;
    mpfr_init2(m_cx, precision);
    mpfr_init2(m_cy, precision);
    mpfr_init2(m_size, precision);
    mpfr_init2(m_jre, precision);
    mpfr_init2(m_jim, precision);
    if (mpfr_set_str(m_cx, cx, 0, GMP_RNDN) || mpfr_set_str(m_cy, cy, 0, GMP_RNDN)
        || mpfr_set_str(m_size, size, 0, GMP_RNDN)) {
        fprintf(stderr, "mdzref: bad coordinate string\n");
        return 0;
    }
    if (family == FAMILY_JULIA) {
        if (mpfr_set_str(m_jre, jre, 0, GMP_RNDN) || mpfr_set_str(m_jim, jim, 0, GMP_RNDN)) {
            fprintf(stderr, "mdzref: bad julia string\n");
            return 0;
        }
    }
    img->use_multi_prec = multi_prec;
    img->use_rounding = rounding;
    if (!set_size(img, w, h, img->aa_factor ? img->aa_factor : 1))
        return 0;
    img->family = family;
    img->fractal = fractal;
    img->depth = depth;
    set_multi_prec(img, multi_prec, rounding);
    coords_set_precision(img->pcoords, precision);
    set_precision(img, precision);
    coords_to(img->pcoords, m_cx, m_cy);
    coords_size(img->pcoords, m_size);
    if (family == FAMILY_JULIA) {
        mpfr_set(img->u.julia.c_re, m_jre, GMP_RNDN);
        mpfr_set(img->u.julia.c_im, m_jim, GMP_RNDN);
    }
    mpfr_clear(m_cx);
    mpfr_clear(m_cy);
    mpfr_clear(m_size);
    mpfr_clear(m_jre);
    mpfr_clear(m_jim);

    /* main.c init_misc -> image_info_set(w, h, aa) */
    if (!set_size(img, w, h, aa))
        return 0;
    /* render.c:34-37 */
    coords_get_rect(img->pcoords, img->xmin, img->xmax, img->ymax, img->width);
    coords_get_rect_gmp(img->pcoords, img->gxmin, img->gxmax, img->gymax, img->gwidth);
    return img;
}

static void destroy_view(image_info* img)
{
    mpfr_clear(img->xmin);
    mpfr_clear(img->xmax);
    mpfr_clear(img->ymax);
    mpfr_clear(img->width);
    mpfr_clear(img->old_cx);
    mpfr_clear(img->old_cy);
    mpfr_clear(img->old_size);
    mpfr_clear(img->u.julia.c_re);
    mpfr_clear(img->u.julia.c_im);
    mpf_clear(img->gxmin);
    mpf_clear(img->gxmax);
    mpf_clear(img->gymax);
    mpf_clear(img->gwidth);
    coords_free(img->pcoords);
    free(img->raw_data);
    free(img);
}

/* Render one frame through rth_* exactly as render_to_file drives it and
 * copy raw_data (real_width * real_height ints) into out_raw.  Returns 1 on
 * success.  *out_seconds is the wall time from rth_ui_start_render until the
 * last row was reported. */
int mdzref_render(int w, int h, int aa, long depth, int family, int fractal,
                  int multi_prec, int rounding, long precision,
                  const char* cx, const char* cy, const char* size,
                  const char* jre, const char* jim, int threads,
                  int* out_raw, double* out_seconds, double* out_rth_seconds)
{
    image_info* img = build_view(w, h, aa, depth, family, fractal, multi_prec,
                                 rounding, precision, cx, cy, size, jre, jim,
                                 threads);
    if (!img)
        return 0;
    rthdata* rth = (rthdata*)img->rth_ptr;
    if (!rth_ui_init(rth))
        return 0;
    double t0 = now_s();
    rth_ui_start_render(rth);
    for (;;) {
        rth_ui_wait_for_line_done(rth);
        int done = rth_process_lines_rendered(rth);
        if (done == -1)
            break;
    }
    double t1 = now_s();
    if (out_rth_seconds)
        *out_rth_seconds = rth_ui_get_render_time(rth);
    /* rth_ui_quit signals start_cond under status_mutex, not start_mutex
     * (src/render_threads.c:449-455): if the watch thread has not reached its
     * pthread_cond_wait yet the wake-up is lost and the join never returns.
     * Give it time to get there first. */
    usleep(20000);
    rth_ui_quit(rth);
    if (out_seconds)
        *out_seconds = t1 - t0;
    memcpy(out_raw, img->raw_data, (size_t)img->real_width * img->real_height * sizeof(int));
    free(rth->data);
    free(rth);
    destroy_view(img);
    return 1;
}

static int dump_mpfr(char* p, size_t room, const char* name, mpfr_srcptr x)
{
    int n = snprintf(p, room, "%s mpfr %ld %d %ld", name, (long)x->_mpfr_prec,
                     (int)x->_mpfr_sign, (long)x->_mpfr_exp);
    long limbs = (x->_mpfr_prec + 63) / 64;
    for (long i = 0; i < limbs && (size_t)n < room; i++)
        n += snprintf(p + n, room - n, " %016lx", (unsigned long)x->_mpfr_d[i]);
    if ((size_t)n < room)
        n += snprintf(p + n, room - n, "\n");
    return n;
}

static int dump_mpf(char* p, size_t room, const char* name, mpf_srcptr x)
{
    int n = snprintf(p, room, "%s mpf %d %d %ld", name, x->_mp_prec, x->_mp_size,
                     (long)x->_mp_exp);
    int limbs = x->_mp_size < 0 ? -x->_mp_size : x->_mp_size;
    for (int i = 0; i < limbs && (size_t)n < room; i++)
        n += snprintf(p + n, room - n, " %016lx", (unsigned long)x->_mp_d[i]);
    if ((size_t)n < room)
        n += snprintf(p + n, room - n, "\n");
    return n;
}

/* Dump the view fields the line callbacks read (img->xmin, xmax, ymax,
 * width, gxmin, gymax, gwidth, u.julia.c_re/c_im) exactly, one per line:
 *   "<name> mpfr <prec> <sign> <exp> <limb0 hex> ..."   (MPFR layout)
 *   "<name> mpf <prec> <size> <exp> <limb0 hex> ..."    (GMP layout)
 * Returns the number of bytes written, or -1. */
int mdzref_view_dump(int w, int h, int aa, long depth, int family, int fractal,
                     int multi_prec, int rounding, long precision,
                     const char* cx, const char* cy, const char* size,
                     const char* jre, const char* jim, char* out, long room)
{
    image_info* img = build_view(w, h, aa, depth, family, fractal, multi_prec,
                                 rounding, precision, cx, cy, size, jre, jim, 1);
    if (!img)
        return -1;
    long n = 0;
    n += dump_mpfr(out + n, room - n, "xmin", img->xmin);
    n += dump_mpfr(out + n, room - n, "xmax", img->xmax);
    n += dump_mpfr(out + n, room - n, "ymax", img->ymax);
    n += dump_mpfr(out + n, room - n, "width", img->width);
    n += dump_mpfr(out + n, room - n, "julia_re", img->u.julia.c_re);
    n += dump_mpfr(out + n, room - n, "julia_im", img->u.julia.c_im);
    n += dump_mpf(out + n, room - n, "gxmin", img->gxmin);
    n += dump_mpf(out + n, room - n, "gymax", img->gymax);
    n += dump_mpf(out + n, room - n, "gwidth", img->gwidth);
    rthdata* rth = (rthdata*)img->rth_ptr;
    free(rth->lines_drawn);
    free(rth->data);
    free(rth);
    destroy_view(img);
    return (int)n;
}

/* One Mandelbrot-family pixel through the reference's own frac_*_mpfr loop,
 * set up as fractal_mpfr_calculate_line does (src/fractal.c:188-233):
 * z0 = c, wre2 = x*x, wim2 = y*y, bail = 4.  c is given as strings parsed at
 * `precision` bits (round to nearest). */
long mdzref_point_mpfr(int fractal, long depth, long precision,
                       const char* c_re_s, const char* c_im_s)
{
    mpfr_t bail, wim, wre, c_im, c_re, wim2, wre2, t1;
    mpfr_init2(bail, precision);
    mpfr_init2(wim, precision);
    mpfr_init2(wre, precision);
    mpfr_init2(c_im, precision);
    mpfr_init2(c_re, precision);
    mpfr_init2(wim2, precision);
    mpfr_init2(wre2, precision);
    mpfr_init2(t1, precision);
    mpfr_set_si(bail, 4, GMP_RNDN);
    mpfr_set_str(c_re, c_re_s, 0, GMP_RNDN);
    mpfr_set_str(c_im, c_im_s, 0, GMP_RNDN);
    mpfr_set(wre, c_re, GMP_RNDN);
    mpfr_set(wim, c_im, GMP_RNDN);
    mpfr_mul(wre2, c_re, c_re, GMP_RNDN);
    mpfr_mul(wim2, c_im, c_im, GMP_RNDN);
    depth_t r;
    switch (fractal) {
    case BURNING_SHIP:
        r = frac_burning_ship_mpfr(depth, bail, wim, wre, c_im, c_re, wim2, wre2, t1);
        break;
    case GENERALIZED_CELTIC:
        r = frac_generalized_celtic_mpfr(depth, bail, wim, wre, c_im, c_re, wim2, wre2, t1);
        break;
    case VARIANT:
        r = frac_variant_mpfr(depth, bail, wim, wre, c_im, c_re, wim2, wre2, t1);
        break;
    default:
        r = frac_mandel_mpfr(depth, bail, wim, wre, c_im, c_re, wim2, wre2, t1);
    }
    mpfr_clear(bail);
    mpfr_clear(wim);
    mpfr_clear(wre);
    mpfr_clear(c_im);
    mpfr_clear(c_re);
    mpfr_clear(wim2);
    mpfr_clear(wre2);
    mpfr_clear(t1);
    return (long)r;
}

/* One Mandelbrot-family pixel through the reference's hardware-float loop
 * (frac_*, src/frac_mandel.c:5-21 etc.) with z0 = c. */
long mdzref_point_hw(int fractal, long depth, double c_re, double c_im)
{
    long double x = c_re, y = c_im;
    depth_t r;
    switch (fractal) {
    case BURNING_SHIP:
        r = frac_burning_ship(depth, y, x, y, x, y * y, x * x);
        break;
    case GENERALIZED_CELTIC:
        r = frac_generalized_celtic(depth, y, x, y, x, y * y, x * x);
        break;
    case VARIANT:
        r = frac_variant(depth, y, x, y, x, y * y, x * x);
        break;
    default:
        r = frac_mandel(depth, y, x, y, x, y * y, x * x);
    }
    return (long)r;
}
