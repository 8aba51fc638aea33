/* Layout-compatible declarations of the MDZ structs that cross the drop-in
 * boundary.
 *
 * libmdzgpu replaces MDZ's render_threads.c + fractal.c, so MDZ's own
 * render.c, coords.c, image_info.c and GUI keep passing their image_info* and
 * rthdata* into it.  The library therefore has to read those structs with
 * the exact field layout MDZ compiles:
 *   image_info      src/image_info.h:63-122
 *   julia_info      src/image_info.h:51-56
 *   rthdata         src/render_threads.h:20-32
 *   mpfr_t / mpf_t  MPFR and GMP public struct layouts (__mpfr_struct,
 *                   __mpf_struct), which MDZ embeds by value.
 * The field names and order below are kept identical on purpose (this is an
 * ABI, not a design choice); the type names carry an mdz_ prefix so that the
 * header can be included next to MDZ's own headers.  A CPU test compares
 * every offset against the reference headers compiled by gcc. */
#ifndef MDZ_ABI_H
#define MDZ_ABI_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* __mpfr_struct: value = sign * 0.d[n-1]...d[0] * 2^exp, n = ceil(prec/64),
 * limbs least significant first, top bit of d[n-1] set when regular.
 * exp == LONG_MIN+1 / +2 / +3 marks zero / NaN / infinity. */
typedef struct mdz_mpfr {
    long prec;
    int sign;
    long exp;
    uint64_t* d;
} mdz_mpfr;

/* __mpf_struct: value = sign(size) * sum_i d[i] * 2^(64*(i - |size| + exp)). */
typedef struct mdz_mpf {
    int prec;
    int size;
    long exp;
    uint64_t* d;
} mdz_mpf;

#define MDZ_MPFR_EXP_ZERO (-0x7fffffffffffffffL)
#define MDZ_MPFR_EXP_NAN (-0x7fffffffffffffffL + 1)
#define MDZ_MPFR_EXP_INF (-0x7fffffffffffffffL + 2)

typedef struct mdz_julia_info {
    mdz_mpfr c_re[1];
    mdz_mpfr c_im[1];
} mdz_julia_info;

typedef struct mdz_image_info {
    mdz_mpfr xmin[1], xmax[1], ymax[1], width[1];
    mdz_mpf gxmin[1], gxmax[1], gymax[1], gwidth[1];
    mdz_mpfr old_cx[1], old_cy[1], old_size[1];
    void* pcoords;
    int64_t depth;
    int thread_count;
    int draw_lines;
    int* raw_data;
    uint32_t* rgb_data;
    int j_pre;
    void* drawing_area;
    void* rnd_pal;
    int real_width;
    int real_height;
    int user_width;
    int user_height;
    double aspect;
    int aa_factor;
    int family;
    int fractal;
    double colour_scale;
    union {
        mdz_julia_info julia;
    } u;
    bool palette_ip;
    bool zoom_new_win;
    bool use_multi_prec;
    bool use_rounding;
    long precision;
    bool multi_prec_init_done;
    void* rth_ptr;
    int lines_drawn;
    bool ui_ref_center;
} mdz_image_info;

struct mdz_rth_private;

typedef struct mdz_rthdata {
    mdz_image_info* img;
    char* lines_drawn;
    int min_line_drawn;
    int line_draw_count;
    int thread_count;
    int check_stop_px;
    struct mdz_rth_private* data;
} mdz_rthdata;

/* FAMILY_* and fractal enums, src/fractal.h:5-21 */
enum { MDZ_FAMILY_MANDEL = 0, MDZ_FAMILY_JULIA = 1 };
enum {
    MDZ_MANDELBROT = 0,
    MDZ_BURNING_SHIP = 1,
    MDZ_GENERALIZED_CELTIC = 2,
    MDZ_VARIANT = 3
};

#ifdef __cplusplus
}
#endif
#endif
