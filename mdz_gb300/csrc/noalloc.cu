// mdzgpu_render_mp_noalloc: the multi-limb render for callers that must not
// allocate device memory.
//
// Who needs it: code that runs where device memory belongs to someone else
// -- a plugin inside an application whose own pool allocator owns the GPU,
// or a render loop that cannot afford cudaMalloc's implicit device-wide
// synchronisation -- and so cannot let libmdzgpu create a context with its
// own buffers (mdzgpu_create / mdzgpu_render_mp_device allocate them on
// first use).  This entry point allocates nothing on the device: the
// caller passes the inputs (host values) and a device output buffer, and the
// kernel's scratch (the fixed-point coordinate tables and the work counters)
// lives in the file-scope array below, one copy per GPU, held from the first
// call until the process exits.
//
// Limits: real frame width + height <= kNoAllocMaxRows (8192 rows and
// columns together) at up to 36 words per number -- 1.13 MiB of scratch.
// Larger frames are rejected with MDZGPU_ERR_ARG.
//
// Sharing: every call on a device uses the same array.  Calls issued to one
// stream are ordered and safe back to back; calls that can overlap on the
// GPU (different streams, or different host threads) race on the array and
// must not be made.
//
// Host blocking: the coordinate tables are built in a temporary host buffer
// and copied from there (pageable memory), so the call may wait until the
// work queued earlier on the stream has finished before it returns.
//
// Set-up: the array's device address is looked up with cudaGetSymbolAddress
// once per CUDA context (keyed by the context's process-unique id, so a
// caller's own non-primary context, or the new primary context after
// cudaDeviceReset, gets its own lookup) while that context is current.  The
// first call in a context does this; make it before capturing any stream
// into a CUDA graph.
#include <cuda.h>

#include <mutex>
#include <vector>

#include "internal.h"

namespace mdz {
namespace {

constexpr int kNoAllocMaxRows = 8192;  // width + height, real pixels
constexpr int kNoAllocMaxWords = 36;
constexpr size_t kSyncBytes = 256;     // FrameSync, padded
constexpr size_t kTableWords = (size_t)(kNoAllocMaxRows + 2) * kNoAllocMaxWords;
constexpr size_t kScratchWords = kSyncBytes / 4 + kTableWords;

// [FrameSync | xs[W][words] | ys[H][words] | julia[2][words]]
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

constexpr int kMaxContexts = 64;
std::mutex g_setup_mutex;
struct ScratchEntry {
    unsigned long long ctx_id;
    void* ptr;
};
ScratchEntry g_scratch_addr[kMaxContexts] = {};
int g_scratch_entries = 0;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int driver_entry_points()
{
    if (g_ctx_get_current && g_ctx_get_id)
        return MDZGPU_OK;
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = qa;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa)
            != cudaSuccess
        || cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb)
            != cudaSuccess
        || qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b) {
        set_error("no-alloc render: the driver does not provide cuCtxGetCurrent / cuCtxGetId");
        return MDZGPU_ERR_CUDA;
    }
    g_ctx_get_current = (CtxGetCurrentFn)a;
    g_ctx_get_id = (CtxGetIdFn)b;
    return MDZGPU_OK;
}

// Device address of g_noalloc_scratch in the current context (looked up once
// per context, with that context current).
int scratch_address(uint32_t** out)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    int rc = driver_entry_points();
    if (rc)
        return rc;
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) {
        set_error("no-alloc render: cuCtxGetCurrent failed");
        return MDZGPU_ERR_CUDA;
    }
    void* ptr = nullptr;
    if (!ctx) {
        // no context yet on this thread: the runtime makes the device's
        // primary context current while it resolves the symbol
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            set_error("no-alloc render: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return MDZGPU_ERR_CUDA;
        }
        if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) {
            set_error("no-alloc render: no current CUDA context");
            return MDZGPU_ERR_CUDA;
        }
    }
    unsigned long long id = 0;
    if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) {
        set_error("no-alloc render: cuCtxGetId failed");
        return MDZGPU_ERR_CUDA;
    }
    for (int i = 0; i < g_scratch_entries; ++i)
        if (g_scratch_addr[i].ctx_id == id) {
            *out = (uint32_t*)g_scratch_addr[i].ptr;
            return MDZGPU_OK;
        }
    if (!ptr) {
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            set_error("no-alloc render: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return MDZGPU_ERR_CUDA;
        }
    }
    // remember it; when the table is full the oldest entry makes room
    if (g_scratch_entries == kMaxContexts) {
        for (int i = 1; i < kMaxContexts; ++i)
            g_scratch_addr[i - 1] = g_scratch_addr[i];
        --g_scratch_entries;
    }
    g_scratch_addr[g_scratch_entries++] = {id, ptr};
    *out = (uint32_t*)ptr;
    return MDZGPU_OK;
}

}  // namespace
}  // namespace mdz

using namespace mdz;

extern "C" int mdzgpu_render_mp_noalloc(const mdzgpu_frame* f, const mdzgpu_mpval* xmin,
                                        const mdzgpu_mpval* ymax, const mdzgpu_mpval* width,
                                        const mdzgpu_mpval* julia_re,
                                        const mdzgpu_mpval* julia_im, int64_t precision,
                                        int32_t words, int32_t* d_counts, void* stream)
{
    if (!f || !d_counts || f->width <= 0 || f->height <= 0 || f->depth < 1
        || f->depth > 0x7fffffffLL) {
        set_error("no-alloc render: bad frame or output buffer");
        return MDZGPU_ERR_ARG;
    }
    if ((long)f->width + f->height > kNoAllocMaxRows) {
        set_error("no-alloc render: width + height = %ld exceeds the %d-row scratch limit",
                  (long)f->width + f->height, kNoAllocMaxRows);
        return MDZGPU_ERR_ARG;
    }
    int w = words > 0 ? words : mp_words_for_precision((long)precision);
    while (w <= kNoAllocMaxWords && !mp_words_supported(w))
        ++w;
    if (w > kNoAllocMaxWords) {
        set_error("no-alloc render: precision %lld needs more than %d words",
                  (long long)precision, kNoAllocMaxWords);
        return MDZGPU_ERR_ARG;
    }
    int device = 0;
    MDZ_CUDA_TRY(cudaGetDevice(&device));
    uint32_t* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc)
        return rc;
    int sms = 0;
    MDZ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));

    // host side: the tables MPFR's coordinate roundings give (as
    // mdzgpu_render_mp computes them)
    const int W = f->width, H = f->height;
    std::vector<uint32_t> tab((size_t)(W + H + 2) * w, 0);
    rc = mpfr_coordinate_tables(xmin, ymax, width, W, 0, H, (long)precision, w, tab.data(),
                                tab.data() + (size_t)W * w);
    if (!rc && f->family == MDZ_FAMILY_JULIA)
        rc = mpfr_round_to_fixed(julia_re, (long)precision, w, tab.data() + (size_t)(W + H) * w)
             | mpfr_round_to_fixed(julia_im, (long)precision, w,
                                   tab.data() + (size_t)(W + H + 1) * w);
    if (rc || (f->family == MDZ_FAMILY_JULIA
               && (!fx_fits_coordinate(tab.data() + (size_t)(W + H) * w, w)
                   || !fx_fits_coordinate(tab.data() + (size_t)(W + H + 1) * w, w)))) {
        set_error("no-alloc render: coordinates must satisfy |x|, |y| < 4");
        return MDZGPU_ERR_RANGE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* tables = scratch + kSyncBytes / 4;
    // the work counters must start at zero on every call
    MDZ_CUDA_TRY(cudaMemsetAsync(scratch, 0, kSyncBytes, s));
    MDZ_CUDA_TRY(cudaMemcpyAsync(tables, tab.data(), tab.size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, s));
    MpLaunch p;
    p.W = W;
    p.H = H;
    p.row0 = 0;
    p.nrows = H;
    p.family = f->family;
    p.fractal = f->fractal;
    p.depth = (uint32_t)f->depth;
    p.words = w;
    p.xs = tables;
    p.ys = tables + (size_t)W * w;
    p.julia = tables + (size_t)(W + H) * w;
    p.out = d_counts;
    p.sync = (FrameSync*)scratch;
    p.tile_rows_done = nullptr;
    p.band_flags = nullptr;
    p.stop = nullptr;
    // launch_mp reads only the SM count from the context
    mdzgpu_ctx shape;
    shape.device = device;
    shape.num_sms = sms;
    rc = launch_mp(&shape, p, s);
    shape.stream = nullptr;
    return rc;
}
