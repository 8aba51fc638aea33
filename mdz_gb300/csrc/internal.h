// Internal declarations shared by the libmdzgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>
#include <vector>

#include "../../include/mdzgpu.h"

namespace mdz {

// Records the calling thread's last error (read by mdzgpu_last_error) and
// prints it to stderr, MDZ's error channel (src/render_threads.c:179).
void set_error(const char* fmt, ...);

#define MDZ_CUDA_TRY(expr)                                                     \
    do {                                                                       \
        cudaError_t _e = (expr);                                               \
        if (_e != cudaSuccess) {                                               \
            ::mdz::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,       \
                             cudaGetErrorString(_e));                          \
            return MDZGPU_ERR_CUDA;                                            \
        }                                                                      \
    } while (0)

// Grows a device allocation to at least `bytes`; never shrinks.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t want);
    void release();
};

// Grows a pinned, device-mapped host allocation.
struct PinnedBuf {
    void* host = nullptr;
    void* dev = nullptr;
    size_t bytes = 0;
    int ensure(size_t want);
    void release();
};

// Per-frame device scratch for the work-queue kernels: tile counter,
// pixel-iteration sum and per-tile-row completion counters.
struct FrameSync {
    unsigned int tile_counter;
    unsigned int pad;
    unsigned long long iter_sum;
};

}  // namespace mdz

namespace mdz {
// Completion of a launch without a stream command behind it (a command
// queued behind a long kernel holds its hardware queue, and the streams
// that share that queue, until the kernel ends): every thread counts
// itself out, the last one stores `value` into a pinned host word that the
// host polls.  `count` is zeroed before the launch.
struct DoneSignal {
    unsigned* count = nullptr;
    volatile int* host = nullptr;
};
#ifdef __CUDACC__
__device__ __forceinline__ void done_signal(const DoneSignal& s, int value)
{
    if (!s.count)
        return;
    __threadfence();
    const unsigned total = gridDim.x * gridDim.y * gridDim.z * blockDim.x * blockDim.y * blockDim.z;
    if (atomicAdd(s.count, 1u) + 1u == total) {
        __threadfence_system();
        *s.host = value;
        __threadfence_system();
    }
}
#endif
}  // namespace mdz

struct mdzgpu_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;   // high priority: the streamed orbit
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_side0 = nullptr;
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;  // around one pixel-pass launch
    mdz::DevBuf counts;     // int32 counts
    mdz::DevBuf sync;       // FrameSync + tile-row counters
    mdz::DevBuf coords;     // fixed-point pixel coordinates (MP path)
    mdz::DevBuf orbit;      // reference orbit (perturbation)
    mdz::DevBuf orbit_fx;   // fixed-point reference state
    mdz::DevBuf aux;        // per-pixel float output (perturbation)
    mdz::DevBuf lists;      // escalation pixel lists (perturbation)
    mdz::PinnedBuf pinned;  // small host-mapped status words
    mdz::PinnedBuf staging; // pinned host copy of counts
    mdz::DevBuf pstate;     // perturbation pixel state between steps (32 B/pixel)
    mdz::DevBuf pqueue;     // step counters + two pixel queues
    mdz::PinnedBuf stepinfo;  // step results read by the host
    mdz::DevBuf palette;    // colouring: up to 256 colours
    // polls a bounded device wait makes before it gives up (mdz::kSpinLimit
    // unless mdzgpu_set_wait_limit changed it)
    int wait_limit = 1 << 25;
    // pixels of the last perturbation render (its escalation lists sit in
    // `lists`); 0 when no list is current
    int64_t esc_pixels = 0;
};

namespace mdz {

// Bounded device waits: ~2^25 polls of >= 256 ns (several seconds), far
// beyond any legitimate wait, then the launch's error flag is raised.
constexpr int kSpinLimit = 1 << 25;

struct Fp64Launch {
    int W, H;           // real frame size
    int row0, nrows;    // rows rendered by this launch
    int family, fractal;
    uint32_t depth;
    double xmin, xmax, ymax, jre, jim;
    int32_t* out;       // out[(line - row0) * W + ix]
    FrameSync* sync;
    unsigned int* tile_rows_done;  // per 4-row band
    volatile int* band_flags;      // host-mapped, per 4-row band (may be null)
    volatile int* stop;            // host-mapped stop word (may be null)
};
int launch_fp64(mdzgpu_ctx* ctx, const Fp64Launch& p, cudaStream_t s);

struct MpLaunch {
    int W, H, row0, nrows;
    int family, fractal;
    uint32_t depth;
    int words;               // 32-bit words per fixed-point number
    const uint32_t* xs;      // [W][words] pixel x coordinates
    const uint32_t* ys;      // [nrows][words] pixel y coordinates
    const uint32_t* julia;   // [2][words] c_re, c_im (julia family)
    int32_t* out;
    FrameSync* sync;
    unsigned int* tile_rows_done;
    volatile int* band_flags;
    volatile int* stop;
    // list mode (perturbation escalation): render only the pixels listed,
    // out[list[i]] with x = xs[list[i] % W], y = ys[list[i] / W]
    const unsigned* list = nullptr;
    const unsigned* list_count = nullptr;
    float* mag = nullptr;   // |z|^2 at escape (FP32), when non-null
    DoneSignal done;        // optional: stores 1 when the launch is complete
                            // (3 when it also reached the list's end)
    // list pass in chunks: this launch takes tiles tile_base + [0, tile_limit)
    unsigned tile_base = 0, tile_limit = 0xffffffffu;
    // polls a bounded wait of the fused launch makes before it gives up
    int spin_limit = kSpinLimit;
};
int launch_mp(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s);
bool mp_words_supported(int words);
// Word counts the multi-limb kernel is compiled for (one translation unit
// each; the build reads this list).
#define MDZ_MP_WORDS_LIST(X) X(4) X(6) X(8) X(10) X(12) X(16) X(20) X(24) X(28) X(34) X(36)
// Word counts beyond one thread's registers: the warp-cooperative kernel
// (mpw_kernel.cu), as (words, lanes per pixel G, 64-bit limbs per lane Q)
// with words = 2 G Q (one translation unit each; the build reads this list).
#define MDZ_MPW_LIST(X) \
    X(48, 8, 3) X(64, 8, 4) X(80, 8, 5) X(96, 8, 6) X(128, 16, 4) X(160, 16, 5) X(192, 16, 6) \
    X(256, 32, 4)
// Largest word count of the one-thread kernel (and of the serving engine's
// multi-limb slice kernels).
constexpr int kMpThreadMaxWords = 36;
template <int N>
int launch_words(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s);
template <int G, int Q>
int launch_wide(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s);
template <int G, int Q>
int preload_wide();
template <int N>
int preload_words();
// Loads (and sets up) every multi-limb frame kernel / every perturbation
// pass kernel now: with lazy module loading the first launch of a kernel
// waits for the work running on the device, which would stall a server
// that launches an escalation pass while others run.
int preload_mp_kernels();
int preload_perturb_kernels();

struct OrbitLaunch {
    int limbs;              // L radix-2^28 signed digits, F = 28 (L - 1)
    const int* c_re;        // [L] centre, balanced signed digits
    const int* c_im;
    int* digits;            // [max_k + 1][2][L] raw digits of every Z_k
    float4* zq;             // [max_k + 1] (Z_k re, im, |Z_k|^2, 0) in FP32
    double2* zd;            // [max_k + 1] Z_k mantissas in FP64 ...
    int* ze;                // ... times 2^ze[k]
    double* dd;             // [max_k + 1] D_k = |Z_k|^2 - 4 = dd * 2^de
    int* de;
    int max_k;              // last index computed (depth + 1)
    int* out_len;           // number of valid entries (device)
    int* sm_busy = nullptr; // serving: producers per SM id (counted while running)
    int sm_words = 0;
    unsigned* tiny = nullptr;  // [max_k / 32 + 2] bit k: |Z_k|^2 < 2^-120 (FP32)
    // [max_k / 32 + 2] bit k: |Z_k|^2 > 4 - 2^-14 or < 2^-60 in FP32 (the
    // entries where the FP32 pixel step needs a test)
    unsigned* att = nullptr;
    // formula: MDZ_MANDELBROT, MDZ_BURNING_SHIP (Im = 2 |Re Im| + Ci) or
    // MDZ_GENERALIZED_CELTIC (Re = |Re^2 - Im^2| + Cr)
    int fractal = 0;
    // burning ship / celtic: the fold quantity F_k (Re Im, or Re^2 - Im^2)
    // = fm * 2^fe, its sign in zq[k].w, and bit k of `axis` set where F_k is
    // within 2^-100 of 0 (a pixel's dz can move it across the fold there)
    double* fm = nullptr;
    int* fe = nullptr;
    unsigned* axis = nullptr;
    // Julia family: Z_0 = (z0_re, z0_im) (the view centre) and c_re / c_im
    // the Julia constant; null: Z_0 = 0 (then Z_1 = C)
    const int* z0_re = nullptr;
    const int* z0_im = nullptr;
    // MDZ_VARIANT (celtic fold on odd iterations, src/frac_variant.c:14-17):
    // the step Z_k -> Z_{k+1} folds when k % 2 == fold_parity
    int fold_parity = 1;
    // polls the finisher's bounded wait for the producer makes before it
    // gives up (sets progress[4])
    int spin_limit = kSpinLimit;
};
int launch_orbit(const OrbitLaunch& p, cudaStream_t s);
int orbit_max_limbs();

struct PerturbLaunch {
    int W, H, row0, nrows;
    uint32_t depth;
    // Julia family (q_len non-null): entries [0, *orbit_len) are the view
    // orbit V (V_0 = centre, no dc term: a pixel starts at V_0 with its
    // offset as delta); entries [q0, q0 + *q_len) the critical orbit Q
    // (Q_0 = 0), which every rebase and the end of either orbit go to.
    // MDZ_VARIANT: [0, *orbit_len) folds at odd steps, [q0, q0 + *q_len)
    // at even steps; a rebase takes the one whose parity matches the
    // pixel's iteration count.
    int q0 = 0;
    const int* q_len = nullptr;
    bool julia = false;     // Julia family (z0 = pixel; see above)
    double hs_m;            // half pixel spacing = hs_m * 2^hs_e, <= 40 bits
    int hs_e;
    const float4* zq;
    const double2* zd;
    const int* ze;
    const double* dd;
    const int* de;
    const int* orbit_len;   // device: valid orbit entries
    const unsigned* tiny;   // bit mask of tiny |Z_k| (see OrbitLaunch)
    const unsigned* att = nullptr;  // attention bit mask (see OrbitLaunch); null: unused
    int fractal = 0;        // MDZ_MANDELBROT / _BURNING_SHIP / _GENERALIZED_CELTIC
    const double* fm = nullptr;  // fold quantity F_k = fm * 2^fe (see OrbitLaunch)
    const int* fe = nullptr;
    const unsigned* axis = nullptr;
    int32_t* out;
    float* mag;             // |z|^2 at escape (may be null)
    FrameSync* sync;
    unsigned long long* rebases;
    volatile int* stop;
    // precision escalation: pixels whose rebases cancelled more than
    // lost_limit bits are appended to flag_out (frame-linear indices)
    float lost_limit = 1e30f;
    unsigned* flag_out = nullptr;
    unsigned* flag_out_count = nullptr;
    const unsigned* list_in = nullptr;        // list pass: pixels to render
    const unsigned* list_in_count = nullptr;
    // fused launch: orbit progress words (device)
    int* raw_len = nullptr;
    int* fin_len = nullptr;
    int* orbit_done = nullptr;
    int* orbit_error = nullptr;
    int* producer_sm = nullptr;  // SM id + 1 of the orbit producer block
    DoneSignal done;             // optional: stores 1 when the launch is complete
                                 // (3 when it also reached the list's end)
    // list pass in chunks: this launch takes tiles tile_base + [0, tile_limit)
    unsigned tile_base = 0, tile_limit = 0xffffffffu;
    // polls a bounded wait of the fused launch makes before it gives up
    int spin_limit = kSpinLimit;
};
// pass 0: FP32 frame pass; pass 1: FP64 pass over list_in
int launch_perturb(mdzgpu_ctx* ctx, const PerturbLaunch& p, cudaStream_t s, int pass);
// The orbit as a cooperative producer + finisher launch that publishes its
// progress: progress[1] digits written, [2] entries finished (in whole
// batches of 256), [3] producer done (final length in *o.out_len), [4] a
// bounded wait gave up, [5] SM id + 1 of the producer while it runs.
// `done` (optional) stores 1 when the launch is complete, 2 if it gave up.
int launch_orbit_stream(const OrbitLaunch& o, int* progress, cudaStream_t s,
                        DoneSignal done = DoneSignal{});
// One step of the FP32 pass over the queue in[0..n) (in == nullptr: every
// pixel of the frame, fresh): pixels read the orbit progress in p (fin_len,
// orbit_done, orbit_len), iterate at most `budget` iterations, and the
// unfinished ones go to out; counters[0] = pull counter, counters[1] = out
// count, counters[2] = working blocks (all reset by the launch).  Blocks
// placed on the orbit producer's SM (p.producer_sm) leave it to the producer.
int launch_perturb_step(int num_sms, const PerturbLaunch& p, const unsigned* in, unsigned n,
                        unsigned* out, unsigned* counters, uint4* state, unsigned budget,
                        cudaStream_t s, cudaEvent_t before = nullptr,
                        cudaEvent_t after = nullptr);
// Orbit + FP32 pixel pass in one cooperative launch (progress words in p).
int launch_fused(mdzgpu_ctx* ctx, const OrbitLaunch& o, const PerturbLaunch& p, cudaStream_t s);

// Colouring epilogue over device counts (palette already on the device).
int launch_colour(mdzgpu_ctx* ctx, const int32_t* d_raw, int real_w, int real_h, int aa,
                  const mdzgpu_palette* pal, const uint32_t* d_palette, uint32_t* d_rgb,
                  cudaStream_t s);

// Fixed-point conversion helpers (host).  A fixed-point number has `words`
// 32-bit words, two's complement, least significant first, and
// F = 32*words - 8 fractional bits.
int fx_from_mpval(const mdzgpu_mpval* v, int words, uint32_t* out);
int fx_from_mpfr(const mdz_mpfr* v, int words, uint32_t* out);
int fx_from_mpf(const mdz_mpf* v, int words, uint32_t* out);
double fx_to_double(const uint32_t* x, int words);
// out = a + sign * (k * step) / div   (k, div > 0), truncated toward -inf
void fx_affine(const uint32_t* a, const uint32_t* step, long k, long div,
               int sign, int words, uint32_t* out);
double mpfr_to_double_rn(const mdz_mpfr* v);
bool fx_fits_coordinate(const uint32_t* x, int words);
// Balanced radix-2^28 digits (L of them, F = 28 (L - 1)) of an mpval.
int digits28_from_mpval(const mdzgpu_mpval* v, int L, int* out);
// Half pixel spacing width / (2 W) rounded to 40 significant bits.
int half_spacing(const mdzgpu_mpval* width, int W, double* hs_m, int* hs_e);
int mp_words_for_precision(long precision);
// Pixel coordinate tables of the MPFR path at precision p: x[ix] for
// ix < W and y[row0 + r] for r < nrows, each the p-bit value
// fractal_mpfr_calculate_line computes, converted to fixed point.
int mpfr_coordinate_tables(const mdzgpu_mpval* xmin, const mdzgpu_mpval* ymax,
                           const mdzgpu_mpval* width, int W, int row0, int nrows, long p,
                           int words, uint32_t* xs, uint32_t* ys);
// A value rounded to p bits (mpfr_set into a p-bit variable), as fixed point.
int mpfr_round_to_fixed(const mdzgpu_mpval* v, long p, int words, uint32_t* out);

// Reference-orbit buffer: byte offsets of its 256-byte aligned pieces for
// `entries` entries of L digits (zf at 0).
struct OrbitLayout {
    size_t zd, ze, dd, de, tiny, fm, fe, axis, att, len, dig, reb, raw, bytes;
};
OrbitLayout orbit_layout(size_t entries, int L);
// Multi-limb word count of the perturbation's last escalation pass.
int perturb_mp_words(long precision);
// Fixed-point pixel coordinates c = centre + ((2 ix - W) hs, (H - 2 line) hs)
// of the perturbation geometry: tab = [x[W] | y[H]] of `words` words each.
int perturb_tables(const mdzgpu_mpval* cx, const mdzgpu_mpval* cy, double hs_m, int hs_e,
                   int W, int H, int words, std::vector<uint32_t>& tab);


}  // namespace mdz
