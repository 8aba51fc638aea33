/* libmdzgpu: GB300 (sm_103a) escape-time renderer for MDZ.
 *
 * Two layers, both plain C ABI (no CUDA or torch types in any signature):
 *
 * 1. Drop-in layer.  The exact entry points of MDZ's render_threads.h and
 *    fractal.h, so an MDZ build links libmdzgpu in place of
 *    render_threads.o + fractal.o and its render.c / coords.c / image_info.c
 *    / palette / GUI code stays unchanged.  rth_ui_start_render renders the
 *    whole frame on the GPU; the callback installed with rth_set_next_line_cb
 *    selects the method exactly as image_info_set_multi_prec does
 *    (src/image_info.c:226-249):
 *        fractal_calculate_line       -> FP64 kernel (bit-exact with MDZ's
 *                                        double build without FMA)
 *        fractal_mpfr_calculate_line  -> multi-limb fixed-point kernel fed
 *                                        from img->xmin/ymax/width (MPFR)
 *        fractal_gmp_calculate_line   -> multi-limb fixed-point kernel fed
 *                                        from img->gxmin/gymax/gwidth (GMP)
 *    Progress is published row by row through the same lines_rendered /
 *    lines_drawn protocol, so render.c's progressive colouring works.
 *
 * 2. Explicit layer (mdzgpu_*).  Frame renders with explicit parameters,
 *    host or device output buffers, and the perturbation method; plus the
 *    serving loop.  Used by the drop-in layer, the tests and bench.py.
 *
 * Errors: functions returning int use 0 = MDZGPU_OK, negative = error,
 * except the drop-in entry points, which keep MDZ's conventions (1 = ok /
 * 0 = fail, NULL on allocation failure, message on stderr).
 * mdzgpu_last_error() returns the calling thread's last message. */
#ifndef MDZGPU_H
#define MDZGPU_H

#include <stddef.h>
#include <stdint.h>

#include "mdz_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Drop-in layer: src/render_threads.h:41-87 and src/fractal.h:42-44.  */
/* ------------------------------------------------------------------ */

/* src/render_threads.h:41 rth_create(): allocates the rthdata and its
 * private state; NULL on allocation failure. */
mdz_rthdata* rth_create(void);

/* src/render_threads.h:43 rth_init(): (re)binds img, allocates the
 * lines_rendered / lines_drawn arrays (user_height entries); 1 ok, 0 fail. */
int rth_init(mdz_rthdata* rth, int thread_count, int line_draw_count,
             mdz_image_info* img);

/* src/render_threads.h:54 rth_ui_init(): starts the watch thread that waits
 * for rth_ui_start_render; 1 ok, 0 fail. */
int rth_ui_init(mdz_rthdata* rth);

/* src/render_threads.h:55-61: start / stop / quit / timing controls. */
void rth_ui_start_render(mdz_rthdata* rth);
void rth_ui_stop_render(mdz_rthdata* rth);
void rth_ui_stop_render_and_wait(mdz_rthdata* rth);
void rth_ui_quit(mdz_rthdata* rth);
void rth_ui_stop_timer(mdz_rthdata* rth);
void rth_ui_wait_until_started(mdz_rthdata* rth);
double rth_ui_get_render_time(mdz_rthdata* rth);

/* src/render_threads.h:70: selects the method (see above). */
void rth_set_next_line_cb(mdz_rthdata* rth,
                          int (*next_line_cb)(mdz_image_info*, int));

/* src/render_threads.h:83-87: progress protocol, cooperative stop. */
int rth_process_lines_rendered(mdz_rthdata* rth);
int rth_render_should_stop(mdz_rthdata* rth);
int rth_ui_wait_for_line_done(mdz_rthdata* rth);

/* src/fractal.h:42-44: render one real row `line` of img->raw_data on the
 * GPU.  Return 1 if rendering should continue, 0 if it was stopped. */
int fractal_calculate_line(mdz_image_info* img, int line);
int fractal_mpfr_calculate_line(mdz_image_info* img, int line);
int fractal_gmp_calculate_line(mdz_image_info* img, int line);

/* ------------------------------------------------------------------ */
/* Explicit layer.                                                     */
/* ------------------------------------------------------------------ */

enum {
    MDZGPU_OK = 0,
    MDZGPU_ERR_ARG = -1,      /* invalid argument */
    MDZGPU_ERR_CUDA = -2,     /* CUDA runtime error */
    MDZGPU_ERR_NOMEM = -3,    /* allocation failed */
    MDZGPU_ERR_RANGE = -4,    /* value outside the fixed-point range */
    MDZGPU_ERR_STOPPED = -5,  /* stopped through the stop word */
    MDZGPU_ERR_TIMEOUT = -6,  /* a bounded device wait gave up */
    MDZGPU_ERR_UNSUPPORTED = -7
};

typedef struct mdzgpu_ctx mdzgpu_ctx;

/* Context = one CUDA device, one stream and the reusable device buffers. */
mdzgpu_ctx* mdzgpu_create(int device);
void mdzgpu_destroy(mdzgpu_ctx* ctx);
const char* mdzgpu_last_error(void);
const char* mdzgpu_version(void);

/* Frame geometry: the REAL (supersampled) size, as img->real_width/height. */
typedef struct mdzgpu_frame {
    int32_t width;
    int32_t height;
    int32_t family;   /* MDZ_FAMILY_MANDEL / MDZ_FAMILY_JULIA */
    int32_t fractal;  /* MDZ_MANDELBROT .. MDZ_VARIANT */
    int64_t depth;    /* maximum iterations, 1 .. INT32_MAX */
} mdzgpu_frame;

/* Filled by every render call (may be NULL). */
typedef struct mdzgpu_stats {
    double kernel_ms;       /* device time of the render kernels (events) */
    double wall_ms;         /* host wall time of the whole call */
    int64_t pixel_iters;    /* sum over pixels of (count ? count : depth) */
    int64_t h2d_bytes;      /* host->device bytes copied by the call */
    int64_t d2h_bytes;      /* device->host bytes copied by the call */
    int32_t launches;       /* kernels launched by the call */
    int32_t words;          /* 32-bit words per fixed-point number (MP) */
    double orbit_ms;        /* reference-orbit kernel time (perturbation) */
    int64_t rebases;        /* rebases taken (perturbation) */
    int64_t orbit_len;      /* reference orbit length (perturbation) */
    int64_t escalated_fp64; /* pixels re-run with FP64 deltas (perturbation) */
    int64_t escalated_mp;   /* pixels re-run on the multi-limb kernel */
    double pixel_ms;        /* device time of the FP32 pixel-pass launches
                               alone (perturbation; events around each) */
    int64_t pixel_launches; /* FP32 pixel-pass launches (perturbation) */
    double esc_fp64_ms;     /* device time of the FP64 escalation pass */
    double esc_mp_ms;       /* device time of the multi-limb escalation pass */
} mdzgpu_stats;

/* An arbitrary-precision binary value with MPFR's meaning:
 *   value = sign * 0.d[n-1] d[n-2] ... d[0] (binary) * 2^exp,
 * limbs least significant first, d[n-1] normalised (top bit set).
 * n == 0 or d == NULL means zero. */
typedef struct mdzgpu_mpval {
    int32_t sign;
    int32_t nlimbs;
    int64_t exp;
    const uint64_t* d;
} mdzgpu_mpval;

/* FP64 path (the fractal_calculate_line arithmetic, src/fractal.c:29-117):
 * width = xmax - xmin; y = ymax - (width/W)*line; x = (ix/W)*width + xmin,
 * each an IEEE double operation with round-to-nearest and no contraction.
 * counts: host buffer of width*height int32 (row-major); a count is the
 * first iteration with |z|^2 > 4, or 0 if not escaped within depth. */
int mdzgpu_render_fp64(mdzgpu_ctx* ctx, const mdzgpu_frame* f, double xmin,
                       double xmax, double ymax, double julia_re,
                       double julia_im, int32_t* counts, mdzgpu_stats* st);
/* Same, output left in device memory (d_counts, width*height int32). */
int mdzgpu_render_fp64_device(mdzgpu_ctx* ctx, const mdzgpu_frame* f,
                              double xmin, double xmax, double ymax,
                              double julia_re, double julia_im,
                              int32_t* d_counts, mdzgpu_stats* st);

/* Multi-limb fixed-point path (fractal_mpfr_calculate_line geometry,
 * src/fractal.c:159-192): x = xmin + ix*width/W, y = ymax - line*width/W.
 * `words` = 32-bit words per number (0 = choose from `precision`: the
 * smallest even count with at least precision+8 bits); the number has
 * 32*words-8 fractional bits.  |coordinates| must be < 4. */
int mdzgpu_render_mp(mdzgpu_ctx* ctx, const mdzgpu_frame* f,
                     const mdzgpu_mpval* xmin, const mdzgpu_mpval* ymax,
                     const mdzgpu_mpval* width, const mdzgpu_mpval* julia_re,
                     const mdzgpu_mpval* julia_im, int64_t precision,
                     int32_t words, int32_t* counts, mdzgpu_stats* st);
int mdzgpu_render_mp_device(mdzgpu_ctx* ctx, const mdzgpu_frame* f,
                            const mdzgpu_mpval* xmin, const mdzgpu_mpval* ymax,
                            const mdzgpu_mpval* width,
                            const mdzgpu_mpval* julia_re,
                            const mdzgpu_mpval* julia_im, int64_t precision,
                            int32_t words, int32_t* d_counts,
                            mdzgpu_stats* st);
/* No counterpart in the reference.  mdzgpu_render_mp without any device
 * allocation, for callers that may not allocate GPU memory (a plugin whose
 * host application's pool allocator owns the device, or a render loop that
 * cannot take cudaMalloc's implicit device synchronisation).  Same inputs and
 * results as mdzgpu_render_mp_device; d_counts is the caller's device buffer
 * of width*height int32; the kernel is queued on `stream` (a cudaStream_t,
 * NULL = default stream).  The coordinate tables are copied from a temporary
 * (pageable) host buffer, so the call may block until the work queued
 * earlier on that stream has finished.  Scratch is a fixed 1.13 MiB array
 * per GPU inside the library, held until the process exits: frames with
 * width + height > 8192 or needing more than 36 words are rejected
 * (MDZGPU_ERR_ARG); a Julia constant outside |x|, |y| < 4 is rejected with
 * MDZGPU_ERR_RANGE, as by mdzgpu_render_mp_device.  Calls on one stream are
 * ordered; calls that may overlap on the GPU (other streams or threads) race
 * on the shared scratch and must not be made.  The first call in each CUDA
 * context (the current one: the device's primary context or the caller's
 * own) looks up the scratch address; make it before capturing a stream. */
int mdzgpu_render_mp_noalloc(const mdzgpu_frame* f, const mdzgpu_mpval* xmin,
                             const mdzgpu_mpval* ymax,
                             const mdzgpu_mpval* width,
                             const mdzgpu_mpval* julia_re,
                             const mdzgpu_mpval* julia_im, int64_t precision,
                             int32_t words, int32_t* d_counts, void* stream);

/* Colouring epilogue (MDZ's palette_apply, src/palette.c:406-463, for
 * aa = 1; do_anti_aliasing, src/render.c:108-158 with get_pixel_colour,
 * src/palette.c:466-503, for aa > 1) on the GPU: raw counts [real_h][real_w]
 * to RGB [real_h/aa][real_w/aa] packed as MDZ packs them (r | g << 8 |
 * b << 16 on little-endian hosts), identical to the reference's colours for
 * 0 <= count * colour_scale + offset < 2^31.  With the _device form the
 * counts never leave the GPU and only the RGB image is copied out. */
typedef struct mdzgpu_palette {
    const uint32_t* colours;  /* host array of `indexes` colours (palette[]) */
    int32_t indexes;          /* pal_indexes, 2..256 */
    int32_t offset;           /* pal_offset */
    double colour_scale;      /* img->colour_scale */
    int32_t interpolate;      /* img->palette_ip */
    int32_t pad;
} mdzgpu_palette;
int mdzgpu_colour(mdzgpu_ctx* ctx, const int32_t* counts, int32_t real_w,
                  int32_t real_h, int32_t aa, const mdzgpu_palette* pal,
                  uint32_t* rgb);
int mdzgpu_colour_device(mdzgpu_ctx* ctx, const int32_t* d_counts,
                         int32_t real_w, int32_t real_h, int32_t aa,
                         const mdzgpu_palette* pal, uint32_t* d_rgb);

/* No counterpart in the reference.  Polls a bounded device wait of this
 * context's perturbation launches makes before it gives up (the orbit
 * finisher waiting for the producer, the fused launch's pixels waiting for
 * finished orbit entries); 0 restores the default (2^25 polls of >= 256 ns,
 * several seconds).  A wait that gives up sets the launch's error word, the
 * kernel returns, and the call reports MDZGPU_ERR_TIMEOUT.  Small values
 * exist to test that path. */
int mdzgpu_set_wait_limit(mdzgpu_ctx* ctx, int32_t polls);

/* No counterpart in the reference.  The pixels (line * W + ix) the last
 * perturbation render on this context re-ran: those its FP32 pass handed to
 * the FP64 pass, and those the FP64 pass handed to the multi-limb kernel, in
 * the order the passes listed them.  Copies at most cap_fp64 / cap_mp indices;
 * *n_fp64 / *n_mp receive the full counts.  Valid until the next
 * perturbation render on the context; MDZGPU_ERR_ARG when there is none. */
int mdzgpu_last_escalations(mdzgpu_ctx* ctx, uint32_t* fp64, int64_t cap_fp64, int64_t* n_fp64,
                            uint32_t* mp, int64_t cap_mp, int64_t* n_mp);

/* Largest `words` value the MP kernel is built for. */
int32_t mdzgpu_mp_max_words(void);

/* Perturbation path (new method; the reference has none).  Renders the
 * Mandelbrot family with the Mandelbrot, burning ship, generalized celtic
 * or variant formula (f->fractal; the folded formulas take |c + d| - |c|
 * from the orbit's exact side of the fold, and an exact FP64 step wherever
 * a pixel can cross it; the variant, whose fold applies on odd iterations
 * only, keeps two orbits, folding at odd and at even steps, and rebases
 * onto the one that matches the pixel's iteration parity) around the
 * centre (cx, cy) with real-axis
 * `width`: pixel (ix, line) is c = (cx + (2 ix - W) hs, cy + (H - 2 line) hs)
 * where hs = width / (2 W) rounded to 40 significant bits (exactly the value
 * mdzgpu_perturb_spacing returns; this is MDZ's centre/size geometry,
 * src/coords.c:265-302, with square pixels).  One reference orbit of the
 * centre is iterated on the GPU in `limbs` radix-2^28 digits (0 = choose
 * from `precision`: ceil(precision / 28) + 1), then every pixel runs in
 * FP32-mantissa / int32-exponent deltas with FP64 rebasing.  counts as in
 * the other paths; mag2 (nullable) receives |z|^2 at escape in FP32, for
 * smooth colouring. */
int mdzgpu_render_perturb(mdzgpu_ctx* ctx, const mdzgpu_frame* f,
                          const mdzgpu_mpval* cx, const mdzgpu_mpval* cy,
                          const mdzgpu_mpval* width, int64_t precision,
                          int32_t limbs, int32_t* counts, float* mag2,
                          mdzgpu_stats* st);
/* Julia family under perturbation (f->family = MDZ_FAMILY_JULIA; MDZ's
 * Julia loop, src/fractal.c:55-59 and :78-88: z0 = the pixel, c = the
 * constant).  Two reference orbits: the view's, from the centre, which the
 * pixels start on with their offset as delta (no dc term), and the
 * critical one, from 0, which every rebase goes to.  No counterpart in the
 * reference (MDZ iterates every pixel in MPFR). */
int mdzgpu_render_perturb_julia(mdzgpu_ctx* ctx, const mdzgpu_frame* f,
                                const mdzgpu_mpval* cx, const mdzgpu_mpval* cy,
                                const mdzgpu_mpval* width,
                                const mdzgpu_mpval* julia_re,
                                const mdzgpu_mpval* julia_im, int64_t precision,
                                int32_t limbs, int32_t* counts, float* mag2,
                                mdzgpu_stats* st);
int mdzgpu_render_perturb_device(mdzgpu_ctx* ctx, const mdzgpu_frame* f,
                                 const mdzgpu_mpval* cx,
                                 const mdzgpu_mpval* cy,
                                 const mdzgpu_mpval* width, int64_t precision,
                                 int32_t limbs, int32_t* d_counts,
                                 float* d_mag2, mdzgpu_stats* st);
/* Half pixel spacing used by the perturbation path: width/(2W) = hs_m 2^hs_e
 * with hs_m in [1, 2) holding at most 40 significant bits. */
int mdzgpu_perturb_spacing(const mdzgpu_mpval* width, int32_t W,
                           double* hs_m, int32_t* hs_e);
/* The reference orbit alone: Z_0 = 0, Z_1 = C, Z_{k+1} = Z_k^2 + C for the
 * centre (cx, cy), iterated on the GPU in `limbs` radix-2^28 digits until
 * |Z_k| > 2 or k = max_k.  Writes *len entries (arrays hold max_k + 1):
 * z_re/z_im = Z_k rounded to double (ldexp-scaled, may underflow), and
 * D_k = |Z_k|^2 - 4 = d_mant * 2^d_exp (exact from the digits when
 * |D_k| < 2^-20).  Any output pointer may be NULL. */
int mdzgpu_reference_orbit(mdzgpu_ctx* ctx, const mdzgpu_mpval* cx,
                           const mdzgpu_mpval* cy, int64_t precision,
                           int32_t limbs, int64_t max_k, double* z_re,
                           double* z_im, double* d_mant, int32_t* d_exp,
                           int64_t* len);

/* The same for the burning ship (Im' = 2 |Re Im| + Ci) and generalized
 * celtic (Re' = |Re^2 - Im^2| + Cr) formulas (`fractal` = MDZ_BURNING_SHIP /
 * MDZ_GENERALIZED_CELTIC; MDZ_MANDELBROT as above). */
int mdzgpu_reference_orbit_formula(mdzgpu_ctx* ctx, int32_t fractal,
                                   const mdzgpu_mpval* cx, const mdzgpu_mpval* cy,
                                   int64_t precision, int32_t limbs, int64_t max_k,
                                   double* z_re, double* z_im, double* d_mant,
                                   int32_t* d_exp, int64_t* len);

/* Orbit digits chosen for a precision (ceil(precision / 28) + 1, >= 5). */
int32_t mdzgpu_perturb_limbs(int64_t precision);

/* Pixel coordinate tables of the multi-limb path: xs[ix] (ix < W) and
 * ys[r] for line row0 + r (r < nrows), each the value
 * fractal_mpfr_calculate_line computes with `precision`-bit MPFR roundings
 * (src/fractal.c:167-186), in the kernel's fixed point (`words` each). */
int mdzgpu_mp_coordinates(const mdzgpu_mpval* xmin, const mdzgpu_mpval* ymax,
                          const mdzgpu_mpval* width, int32_t W, int32_t row0,
                          int32_t nrows, int64_t precision, int32_t words,
                          uint32_t* xs, uint32_t* ys);

/* Fixed-point helpers exposed for tests: convert an mpval to the kernel's
 * fixed-point words (out has `words` entries); 0 ok, MDZGPU_ERR_RANGE. */
int mdzgpu_fx_from_mpval(const mdzgpu_mpval* v, int32_t words, uint32_t* out);

/* Measured pipe throughput of `device` in operations per second, the
 * roofline denominators of these compute-bound kernels: kind 0 = FP32 FFMA,
 * 1 = INT32 IMAD (mad.lo.u32), 2 = FP64 DMUL/DADD (unfused). */
int mdzgpu_measure_peak(int device, int kind, double* ops_per_s);

/* Writes offsetof() of every mdz_image_info / mdz_rthdata field, in
 * declaration order, into out (capacity n); returns the count written.
 * Used to check the drop-in ABI against MDZ's own headers. */
int mdzgpu_abi_layout(int64_t* out, int n);

/* ---- Serving engine (new; the reference renders one image at a time) ----
 *
 * A server owns one GPU and renders many requests at once.  Requests are
 * admitted in arrival order while a slot, device memory (`arena_bytes`),
 * pinned result staging (`staging_bytes`) and work-queue room are free; an
 * admitted request's pixels join a work queue shared with every other
 * admitted request of the same method, and each engine step (one CUDA-graph
 * launch) advances every queued pixel by a bounded number of iterations, so
 * requests that arrive while others run start at the next step and finish
 * independently.  Results are bit-identical to rendering the request alone. */
typedef struct mdzgpu_server mdzgpu_server;

enum {
    MDZGPU_METHOD_AUTO = 0,       /* perturbation for the Mandelbrot, burning
                                     ship and generalized celtic formulas,
                                     multi-limb otherwise */
    MDZGPU_METHOD_PERTURB = 1,    /* as mdzgpu_render_perturb */
    MDZGPU_METHOD_MULTI_LIMB = 2  /* multi-limb fixed point, perturbation
                                     geometry, every formula */
};

enum {
    MDZGPU_REQ_QUEUED = 0,
    MDZGPU_REQ_RUNNING = 1,
    MDZGPU_REQ_DONE = 2,
    MDZGPU_REQ_FAILED = 3,
    MDZGPU_REQ_CANCELLED = 4,
    MDZGPU_REQ_TIMEOUT = 5
};

typedef struct mdzgpu_serve_config {
    int32_t device;
    int32_t max_requests;         /* admitted at once, 1..64 (0 = 64) */
    int64_t arena_bytes;          /* device memory for requests (0 = 8 GiB) */
    int64_t staging_bytes;        /* pinned host memory for results (0 = 512 MiB) */
    int64_t queue_pixels;         /* pixels in flight per method (0 = 2^24) */
    double step_ms;               /* target duration of one step (0 = 2 ms) */
    const char* log_path;         /* JSON line per finished request, or NULL */
} mdzgpu_serve_config;

/* A render request.  Geometry as mdzgpu_render_perturb: centre (cx, cy),
 * real-axis width, square pixels.  The mpval limbs are copied by submit.
 * counts (width*height int32) and mag2 (nullable, float) are host buffers
 * that must stay valid until the request leaves the RUNNING state. */
typedef struct mdzgpu_request {
    int32_t width, height;
    int32_t family, fractal;      /* MDZ_FAMILY_MANDEL / _JULIA; any MDZ formula */
    int64_t depth;
    int64_t precision;
    mdzgpu_mpval cx, cy, span;
    int32_t method;               /* MDZGPU_METHOD_* */
    int32_t pad;
    double timeout_ms;            /* from submission; 0 = none */
    int32_t* counts;
    float* mag2;
    /* Julia family: the constant c (z0 is the pixel); the multi-limb kernel
     * serves it (MDZGPU_METHOD_AUTO picks it) */
    mdzgpu_mpval julia_re, julia_im;
} mdzgpu_request;

typedef struct mdzgpu_request_status {
    int32_t state;                /* MDZGPU_REQ_* */
    int32_t error;                /* MDZGPU_ERR_* when FAILED */
    int32_t method;               /* method used */
    int32_t words;                /* orbit digits (perturbation) or words */
    double queue_ms;              /* submission -> admission */
    double latency_ms;            /* submission -> results in counts */
    int64_t pixel_iters;          /* sum over pixels of (count ? count : depth) */
    int64_t escalated_fp64, escalated_mp, rebases;
    int64_t steps;                /* engine steps the request took part in */
    double main_ms;               /* submission -> main pass finished */
    double esc_wait_ms;           /* main pass -> escalation passes started */
    double esc_ms;                /* escalation passes (0 when none ran) */
} mdzgpu_request_status;

typedef struct mdzgpu_serve_stats {
    int64_t submitted, completed, failed, cancelled, timed_out;
    int64_t steps;                /* engine steps (graph launches) */
    int64_t launches;             /* kernels launched by the engine */
    int64_t pixel_iters;          /* over completed requests */
    double busy_ms;               /* wall time with work on the GPU */
    double latency_p50_ms, latency_p99_ms, latency_max_ms;
    int64_t device_bytes_in_use, device_bytes_peak;
} mdzgpu_serve_stats;

/* NULL on failure (mdzgpu_last_error). */
mdzgpu_server* mdzgpu_serve_create(const mdzgpu_serve_config* cfg);
/* Stops the engine: running requests are cancelled, then everything freed. */
void mdzgpu_serve_destroy(mdzgpu_server* s);
/* Queues a request; *id identifies it.  MDZGPU_ERR_NOMEM if it can never fit
 * the server's memory, MDZGPU_ERR_ARG / _RANGE / _UNSUPPORTED for a bad
 * request. */
int mdzgpu_serve_submit(mdzgpu_server* s, const mdzgpu_request* r, int64_t* id);
/* Current status (any state). */
int mdzgpu_serve_poll(mdzgpu_server* s, int64_t id, mdzgpu_request_status* out);
/* Waits until the request leaves QUEUED/RUNNING or timeout_ms passes
 * (< 0 = no limit); MDZGPU_ERR_TIMEOUT if it did not. */
int mdzgpu_serve_wait(mdzgpu_server* s, int64_t id, double timeout_ms,
                      mdzgpu_request_status* out);
/* Cancels a queued or running request (its buffers are not written after
 * the call's effect is seen in poll). */
int mdzgpu_serve_cancel(mdzgpu_server* s, int64_t id);
/* Forgets a finished request's record (ids of finished requests otherwise
 * stay pollable). */
int mdzgpu_serve_release(mdzgpu_server* s, int64_t id);
int mdzgpu_serve_get_stats(mdzgpu_server* s, mdzgpu_serve_stats* out);
/* Device and pinned-host bytes a request needs while admitted (no GPU
 * needed); MDZGPU_ERR_* for a request the server would refuse. */
int mdzgpu_serve_footprint(const mdzgpu_request* r, int64_t* device_bytes,
                           int64_t* host_bytes);

#ifdef __cplusplus
}
#endif
#endif
