/* Driver for the UNMODIFIED MDZ colouring and settings-file code
 * (TEST INFRASTRUCTURE, oracle).
 *
 * Compiled by oracle/build_ref.sh with MDZ's own src/palette.c,
 * src/render.c, src/image_info.c, src/mdzfileio.c, src/setting.c,
 * src/globals.c, src/cmdline.c and the hot-path sources into
 * oracle/_ref/libmdzref_io.so.  Nothing in the product links it.
 *
 *   mdzref_io_colour  palette_apply (src/palette.c:406-463) for aa = 1 and
 *                     do_anti_aliasing (src/render.c:108-158, through
 *                     get_pixel_colour, src/palette.c:466-503) for aa > 1,
 *                     row by row as render_to_file calls them.
 *   mdzref_io_load    main.c's headless sequence: image_info_create,
 *                     image_info_load_all (settings + palette sections),
 *                     the size logic of init_misc (src/main.c, restated
 *                     below because main.c holds main()), image_info_set,
 *                     then coords_get_rect as render_to_file does; dumps
 *                     the view the line callbacks would read. */
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cmdline.h"
#include "coords.h"
#include "image_info.h"
#include "mdzfileio.h"
#include "palette.h"
#include "render.h"
#include "fractal.h"

/* my_png.c needs libpng; the paths driven here never save an image */
void save_png_file(image_info* img, char* filename)
{
    (void)img;
    (void)filename;
}
void my_png_reset_last_used_filename(void) {}

int mdzref_io_colour(const int* raw, int real_w, int real_h, int aa, int ip, double sc,
                     const uint32_t* pal, int pal_n, int pal_off, uint32_t* rgb)
{
    image_info img;
    memset(&img, 0, sizeof img);
    if (aa < 1 || real_w % aa || real_h % aa || pal_n < 2 || pal_n > 256)
        return 0;
    img.aa_factor = aa;
    img.palette_ip = ip;
    img.colour_scale = sc;
    img.real_width = real_w;
    img.real_height = real_h;
    img.user_width = real_w / aa;
    img.user_height = real_h / aa;
    img.raw_data = (int*)raw;
    img.rgb_data = rgb;
    guint32 local[256];
    memcpy(local, pal, (size_t)pal_n * sizeof(guint32));
    guint32* saved = palette;
    palette = local;
    pal_indexes = pal_n;
    pal_offset = pal_off;
    for (int y = 0; y < img.user_height; ++y) {
        if (aa == 1)
            palette_apply(&img, 0, y, img.user_width, 1);
        else
            do_anti_aliasing(&img, 0, y, img.user_width, 1);
    }
    palette = saved;
    return 1;
}

static int dump_hex(char* p, size_t room, const char* name, mpfr_srcptr x)
{
    mpfr_exp_t e = 0;
    char* s = mpfr_get_str(NULL, &e, 16, 0, x, GMP_RNDN);
    int n;
    if (!s)
        return snprintf(p, room, "%s ?\n", name);
    if (mpfr_zero_p(x))
        n = snprintf(p, room, "%s 0x0p+0 %ld\n", name, (long)mpfr_get_prec(x));
    else if (s[0] == '-')
        n = snprintf(p, room, "%s -0x0.%sp%ld %ld\n", name, s + 1, (long)(4 * e),
                     (long)mpfr_get_prec(x));
    else
        n = snprintf(p, room, "%s 0x0.%sp%ld %ld\n", name, s, (long)(4 * e),
                     (long)mpfr_get_prec(x));
    mpfr_free_str(s);
    return n;
}

/* width / height / aa: the command-line -W / -H / -a values (0 = unset),
 * applied as init_misc does.  Writes the loaded view into `out` as lines
 * "key value" and the palette into pal (256 entries). */
int mdzref_io_load(const char* path, int width, int height, int aa, char* out, long room,
                   uint32_t* pal, int* pal_n, int* pal_off)
{
    static random_palette rnd;
    static guint32 pal_store[256];
    memset(pal_store, 0, sizeof pal_store);
    palette = pal_store;
    pal_indexes = 256;
    pal_offset = 0;
    image_info* img = image_info_create(FAMILY_MANDEL, MANDELBROT);
    if (!img)
        return 0;
    img->rnd_pal = &rnd;
    if (!image_info_load_all(img, MDZ_FRACTAL_SETTINGS | MDZ_PALETTE_DATA, path))
        return 0;
    /* init_misc (src/main.c), with opts.aspect unset */
    int w = width, h = height;
    if (!w && !h) {
        w = img->user_width;
        h = img->user_height;
    } else if (!w) {
        w = h * img->aspect;
    } else if (!h) {
        h = w / img->aspect;
    }
    if (!aa)
        aa = 1;
    image_info_set(img, w, h, aa);
    coords_get_rect(img->pcoords, img->xmin, img->xmax, img->ymax, img->width);
    long n = 0;
    n += snprintf(out + n, room - n,
                  "family %d\nfractal %d\ndepth %ld\nuser_width %d\nuser_height %d\n"
                  "aa %d\nprecision %ld\nmulti_prec %d\nrounding %d\ncolour_scale %.17g\n"
                  "palette_ip %d\n",
                  img->family, img->fractal, (long)img->depth, img->user_width,
                  img->user_height, img->aa_factor, (long)img->precision,
                  img->use_multi_prec, img->use_rounding, img->colour_scale, img->palette_ip);
    n += dump_hex(out + n, room - n, "xmin", img->xmin);
    n += dump_hex(out + n, room - n, "xmax", img->xmax);
    n += dump_hex(out + n, room - n, "ymax", img->ymax);
    n += dump_hex(out + n, room - n, "width", img->width);
    n += dump_hex(out + n, room - n, "julia_re", img->u.julia.c_re);
    n += dump_hex(out + n, room - n, "julia_im", img->u.julia.c_im);
    memcpy(pal, palette, 256 * sizeof(uint32_t));
    *pal_n = pal_indexes;
    *pal_off = pal_offset;
    return (int)n;
}
