// Device-side layout of the serving engine (continuous batching of render
// requests) shared by its kernels and its host loop.
//
// Every admitted request owns a slot.  Its pixels live in a per-method work
// queue as 32-bit entries [slot:6 | fresh:1 | pixel:25]; one step of the
// engine runs each method's slice kernel over the entries of queue `cur`:
// a pixel iterates at most budget[slot] iterations, then either finishes
// (count written, remaining[slot] decremented) or saves its state and is
// appended to queue 1 - cur.  Warps take 32 consecutive entries, so pixels
// of different requests share a warp and finished pixels leave the queue at
// every step (the uneven iteration counts are compacted away).
#pragma once

#include "internal.h"

namespace mdz {

constexpr int kServeSlots = 64;
// method classes: 0 / 1 / 2 = perturbation FP32 pass of the Mandelbrot,
// burning ship and generalized celtic formulas; 3.. = multi-limb kernels in
// MDZ_MP_WORDS_LIST order
#define MDZ_COUNT_ONE(n) +1
constexpr int kServeMpClasses = 0 MDZ_MP_WORDS_LIST(MDZ_COUNT_ONE);
#undef MDZ_COUNT_ONE
constexpr int kServePerturbClasses = 3;
constexpr int kServeClasses = kServePerturbClasses + kServeMpClasses;
constexpr unsigned kEntrySlotShift = 26;
constexpr unsigned kEntryFresh = 1u << 25;
constexpr unsigned kEntryPixelMask = kEntryFresh - 1u;
constexpr long kServeMaxPixels = (long)kEntryPixelMask + 1;
constexpr int kServeSmWords = 1024;   // orbit producers per SM id

// Written by the host before every step (one small copy).
struct ServeCtl {
    unsigned cur;                    // queue read this step
    unsigned pad;
    unsigned long long cancel;       // bit per slot: drop its pixels
    unsigned budget[kServeSlots];    // iterations per pixel this step
};

// Read back by the host after every step (one small copy).
struct ServeStatus {
    unsigned qcount[kServeClasses][2];
    unsigned remaining[kServeSlots];  // pixels of the main pass not finished
    // per class and step parity: first block start, last warp end of the
    // slice kernel (globaltimer ns; ~0 / 0 when the class had no work);
    // the host scales its budgets so that each class's kernel takes one step
    unsigned long long tk[2][kServeClasses][2];
    unsigned long long tstep[2][2];   // per parity: step begin, step end (ns)
    unsigned flagged[kServeSlots];    // perturbation: pixels the FP32 pass flagged so far
};

// Per-slot request description (device copy).
struct ServeReq {
    PerturbLaunch pl;         // geometry, depth, outputs; perturbation: orbit,
                              // escalation list of the FP32 pass
    const uint32_t* xs;       // multi-limb: [W][words] pixel x
    const uint32_t* ys;       // multi-limb: [H][words] pixel y
    int fractal;              // multi-limb formula (MDZ_MANDELBROT ...)
    const uint32_t* julia;    // multi-limb, Julia family: [2][words] c; else null
    int words;
    uint4* state;             // resumable per-pixel state, indexed by pixel
    unsigned state_stride;    // uint4 per pixel
    unsigned pad;
};

struct ServeDev {
    ServeCtl ctl;
    ServeStatus status;
    unsigned qpull[kServeClasses];           // work counter of this step
    unsigned qworkers[kServeClasses];        // blocks draining the queue this step
    unsigned* queue[kServeClasses][2];
    int sm_busy[kServeSmWords];              // orbit producers running per SM
    ServeReq req[kServeSlots];
};

#ifdef __CUDACC__
// Block-uniform: true when this block should leave because a reference
// orbit runs on its SM and another block of the launch already works class
// `cls` (that block drains the queue).  Otherwise the block registers as a
// worker.  Called by every thread of the block at its start.
__device__ __forceinline__ bool serve_block_leaves(ServeDev* d, int cls)
{
    __shared__ int s_leave;
    if (threadIdx.x == 0) {
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        const bool busy = *(volatile const int*)(d->sm_busy + smid % (unsigned)kServeSmWords) > 0;
        const bool others = *(volatile const unsigned*)(d->qworkers + cls) > 0u;
        s_leave = busy && others;
        if (!s_leave)
            atomicAdd(d->qworkers + cls, 1u);
    }
    __syncthreads();
    return s_leave != 0;
}
#endif

#ifdef __CUDACC__
// Records the slice kernel's time span of this step in status.tk (see
// ServeStatus): constructed after serve_block_leaves, ends with the thread.
struct ServeClassTimer {
    unsigned long long* t;
    bool on;
    __device__ static unsigned long long now()
    {
        unsigned long long v;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
        return v;
    }
    __device__ ServeClassTimer(ServeDev* d, int cls, unsigned cur, unsigned n)
        : t(d->status.tk[cur][cls]), on(n != 0u)
    {
        if (on && threadIdx.x == 0)
            atomicMin(t, now());
    }
    __device__ ~ServeClassTimer()
    {
        if (on && (threadIdx.x & 31) == 0)
            atomicMax(t + 1, now());
    }
};
#endif

__host__ __device__ inline unsigned serve_entry(int slot, bool fresh, unsigned pixel)
{
    return ((unsigned)slot << kEntrySlotShift) | (fresh ? kEntryFresh : 0u) | pixel;
}

// Slice kernels (one launch per step each; an empty queue exits at once).
// A block placed on an SM where a reference orbit runs leaves at once, but
// only when another block of the same launch already works the queue: a
// working block pulls until the queue is empty, so no entry is left behind.
int launch_serve_perturb(ServeDev* d, int formula, int num_sms, cudaStream_t s);
int launch_serve_mp(ServeDev* d, int mp_class, int num_sms, cudaStream_t s);
template <int N>
int launch_serve_mp_words(ServeDev* d, int mp_class, int num_sms, cudaStream_t s);
// Appends pixels [0, npix) of `slot` as fresh entries to queue `q` of `cls`.
int launch_serve_enqueue(ServeDev* d, int cls, int q, int slot, unsigned npix, cudaStream_t s);
// End of a step: queue `cur` is consumed; clear its count and the pull counters.
int launch_serve_step_end(ServeDev* d, cudaStream_t s);
// Start of a step: stamps status.tstep[cur][0].
int launch_serve_step_begin(ServeDev* d, cudaStream_t s);
// Word count of multi-limb class cls (kServePerturbClasses ..), 0 if none.
int serve_mp_class_words(int cls);
// Uint4 words of resumable state per pixel of the multi-limb slice kernel.
inline unsigned serve_mp_state_stride(int words)
{
    return (unsigned)((2 * words + 2 + 3) / 4);
}

}  // namespace mdz
