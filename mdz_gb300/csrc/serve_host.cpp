// Serving engine, host side: request preparation, admission by memory
// footprint, the step loop (one CUDA-graph launch per step) and completion.
//
// Life of a request:
//   submit (caller's thread): validate, compute the orbit centre digits or
//     the fixed-point pixel coordinates, footprint; queue it.
//   admit (engine thread, arrival order): a slot, a piece of the device arena,
//     a piece of the pinned staging arena and work-queue room; copy the
//     inputs; perturbation: launch its streamed reference orbit on the
//     slot's high-priority stream and enqueue its pixels at once (they
//     iterate up to the last finished orbit entry); multi-limb: enqueue its
//     pixels.
//   steps: every queued pixel of every request advances by at most its
//     request's budget of iterations (budgets give each running request an
//     equal share of the step, scaled by the measured slice-kernel times).
//   all pixels finished -> perturbation with flagged pixels: the FP64 and
//     multi-limb escalation passes, in chunks on one of the low-priority
//     esc streams (one request at a time on each); then, once the orbit
//     launch has ended too,
//     the results are copied to pinned staging, then to the caller's
//     buffers; the request's memory is released.  The long kernels (orbit,
//     passes) report their end in pinned host words: nothing is queued
//     behind them on any stream.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"
#include "serve.h"

namespace mdz {
namespace {

double wall_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

constexpr size_t kAlign = 256;
constexpr int kEscShare = 2;       // escalation passes use 1 / kEscShare of the SMs
constexpr int kEscLanes = 2;       // requests whose escalation passes run at once
constexpr unsigned kEscTilesPerSm = 32;  // list tiles (32 pixels) per SM and chunk
inline size_t al(size_t b)
{
    return (b + kAlign - 1) & ~(kAlign - 1);
}

// First-fit allocator of byte ranges in [0, size), 256-byte granules,
// neighbouring free ranges merged on release.
class Arena {
public:
    void reset(size_t size)
    {
        size_ = size;
        used_ = 0;
        free_.clear();
        if (size)
            free_[0] = size;
    }
    bool alloc(size_t bytes, size_t* off)
    {
        bytes = al(bytes ? bytes : 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes)
                continue;
            *off = it->first;
            const size_t rest = it->second - bytes, at = it->first + bytes;
            free_.erase(it);
            if (rest)
                free_[at] = rest;
            used_ += bytes;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = al(bytes ? bytes : 1);
        used_ -= bytes;
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + bytes == next->first) {
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += bytes;
                return;
            }
        }
        free_[off] = bytes;
    }
    size_t size() const { return size_; }
    size_t used() const { return used_; }

private:
    size_t size_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;
};

// After the main pass: kEscWait (queued for the escalation passes),
// kEscFp64 / kEscMp (that pass in flight), kCopyWait (result copies wait
// for the orbit launch to end), kFinishing (copies in flight).
enum Phase { kQueued, kRunning, kEscWait, kEscFp64, kEscMp, kCopyWait, kFinishing, kEnded };

// Offsets of a request's pieces in its device block and its pinned block.
struct Layout {
    size_t counts, mag, state, lists, sync, orbit, tables, dev_bytes;
    size_t h_tables, h_digits, h_counts, h_mag, h_misc, host_bytes;
    OrbitLayout ol;
};

struct Req {
    int64_t id = 0;
    int W = 0, H = 0, fractal = 0;
    uint32_t depth = 0;
    long precision = 0;
    int method = 0;        // MDZGPU_METHOD_PERTURB / _MULTI_LIMB
    int cls = 0;           // work-queue class
    int words = 0;         // multi-limb words (perturbation: escalation pass)
    int limbs = 0;         // orbit digits (perturbation)
    size_t npix = 0;
    bool want_mag = false;
    bool julia = false;           // Julia family (multi-limb): c follows the tables
    int32_t* out_counts = nullptr;
    float* out_mag = nullptr;
    double timeout_ms = 0;
    std::vector<int> digits;
    double hs_m = 0;
    int hs_e = 0;
    std::vector<uint32_t> tables;
    Layout lay{};
    size_t dev_off = 0, host_off = 0;
    int slot = -1;
    Phase phase = kQueued;
    // public status (guarded by the server mutex)
    int state = MDZGPU_REQ_QUEUED;
    int error = 0;
    bool cancel = false;
    int cancel_state = MDZGPU_REQ_CANCELLED;
    double t_submit = 0, t_admit = 0, t_done = 0;
    // main pass finished; escalation passes started / ended (0: none)
    double t_main = 0, t_esc0 = 0, t_esc1 = 0;
    int64_t pixel_iters = 0, esc_fp64 = 0, esc_mp = 0, rebases = 0, steps = 0;
    cudaEvent_t ev_done = nullptr;
    unsigned flagged = 0;        // pixels the FP32 pass sent to the escalation passes
    unsigned esc_base = 0;       // escalation pass: list tiles launched so far
    int esc_lane = 0;            // escalation stream it runs on
    bool orbit_running = false;  // streamed orbit not yet complete
    bool cancelled = false;      // finishing only to release the memory
};

Layout make_layout(const Req& r)
{
    Layout l{};
    const size_t n = r.npix;
    size_t o = 0;
    l.counts = o;
    o += al(n * 4);
    l.mag = o;
    if (r.want_mag)
        o += al(n * 4);
    l.state = o;
    if (r.method == MDZGPU_METHOD_PERTURB)
        o += al(n * 32);
    else
        o += al(n * (size_t)serve_mp_state_stride(r.words) * 16);
    l.lists = o;
    if (r.method == MDZGPU_METHOD_PERTURB)
        o += al(256 + 2 * n * 4);
    l.sync = o;
    o += 256;
    l.orbit = o;
    if (r.method == MDZGPU_METHOD_PERTURB) {
        l.ol = orbit_layout((size_t)r.depth + 2, r.limbs);
        o += al(l.ol.bytes);
    }
    l.tables = o;
    o += al(r.tables.size() * 4);
    l.dev_bytes = o;
    size_t h = 0;
    l.h_tables = h;
    h += al(r.tables.size() * 4);
    l.h_digits = h;
    h += al(2 * (size_t)r.limbs * 4 + 4);
    l.h_counts = h;
    h += al(n * 4);
    l.h_mag = h;
    if (r.want_mag)
        h += al(n * 4);
    l.h_misc = h;
    h += 256;
    l.host_bytes = h;
    return l;
}

// Validates a request and computes everything the GPU will need.
int prepare(const mdzgpu_request* q, Req& r)
{
    if (!q) {
        set_error("serve: null request");
        return MDZGPU_ERR_ARG;
    }
    if (q->width <= 0 || q->height <= 0
        || (long)q->width * q->height > kServeMaxPixels) {
        set_error("serve: %d x %d pixels outside (0, %ld]", q->width, q->height,
                  kServeMaxPixels);
        return MDZGPU_ERR_ARG;
    }
    if (q->depth < 1 || q->depth > 0x7ffffffeLL) {
        set_error("serve: depth %lld outside [1, 2^31 - 2]", (long long)q->depth);
        return MDZGPU_ERR_ARG;
    }
    if (q->family != MDZ_FAMILY_MANDEL && q->family != MDZ_FAMILY_JULIA) {
        set_error("serve: unknown family %d", q->family);
        return MDZGPU_ERR_ARG;
    }
    if (q->fractal < MDZ_MANDELBROT || q->fractal > MDZ_VARIANT) {
        set_error("serve: unknown formula %d", q->fractal);
        return MDZGPU_ERR_ARG;
    }
    if (q->precision < 1 || q->precision > 1 << 20) {
        set_error("serve: precision %lld", (long long)q->precision);
        return MDZGPU_ERR_ARG;
    }
    int method = q->method;
    // perturbation for the Mandelbrot, burning ship and celtic formulas; the
    // hybrid (its formula alternates per iteration) on the multi-limb kernel
    // (and the Julia family, z0 = pixel, on the multi-limb kernel)
    if (method == MDZGPU_METHOD_AUTO)
        method = q->fractal == MDZ_VARIANT || q->family == MDZ_FAMILY_JULIA
                     ? MDZGPU_METHOD_MULTI_LIMB
                     : MDZGPU_METHOD_PERTURB;
    if (method != MDZGPU_METHOD_PERTURB && method != MDZGPU_METHOD_MULTI_LIMB) {
        set_error("serve: unknown method %d", q->method);
        return MDZGPU_ERR_ARG;
    }
    if (method == MDZGPU_METHOD_PERTURB && q->fractal == MDZ_VARIANT) {
        set_error("serve: perturbation is not implemented for the mandel-celtic hybrid");
        return MDZGPU_ERR_UNSUPPORTED;
    }
    if (method == MDZGPU_METHOD_PERTURB && q->family == MDZ_FAMILY_JULIA) {
        set_error("serve: perturbation serves the Mandelbrot family only");
        return MDZGPU_ERR_UNSUPPORTED;
    }
    if (!q->counts) {
        set_error("serve: null counts buffer");
        return MDZGPU_ERR_ARG;
    }
    r.W = q->width;
    r.H = q->height;
    r.fractal = q->fractal;
    r.depth = (uint32_t)q->depth;
    r.precision = (long)q->precision;
    r.method = method;
    r.npix = (size_t)q->width * q->height;
    r.want_mag = q->mag2 != nullptr;
    r.out_counts = q->counts;
    r.out_mag = q->mag2;
    r.timeout_ms = q->timeout_ms;
    const int w_need = mp_words_for_precision(r.precision);
    r.words = perturb_mp_words(r.precision);
    if (method == MDZGPU_METHOD_MULTI_LIMB && w_need > kMpThreadMaxWords) {
        set_error("serve: precision %ld needs %d words, the multi-limb slice kernel has %d",
                  r.precision, w_need, kMpThreadMaxWords);
        return MDZGPU_ERR_UNSUPPORTED;
    }
    if (method == MDZGPU_METHOD_PERTURB) {
        r.cls = r.fractal;   // perturbation classes are indexed by formula
        r.limbs = mdzgpu_perturb_limbs(r.precision);
        if (r.limbs < 5 || r.limbs > orbit_max_limbs()) {
            set_error("serve: %d orbit digits outside [5, %d]", r.limbs, orbit_max_limbs());
            return MDZGPU_ERR_UNSUPPORTED;
        }
        r.digits.assign(2 * (size_t)r.limbs, 0);
        if (digits28_from_mpval(&q->cx, r.limbs, r.digits.data())
            || digits28_from_mpval(&q->cy, r.limbs, r.digits.data() + r.limbs)
            || abs(r.digits[r.limbs - 1]) >= 4 || abs(r.digits[2 * r.limbs - 1]) >= 4) {
            set_error("serve: centre must satisfy |cx|, |cy| < 4");
            return MDZGPU_ERR_RANGE;
        }
    } else {
        r.cls = 0;
        for (int c = kServePerturbClasses; c < kServeClasses; ++c)
            if (serve_mp_class_words(c) == r.words)
                r.cls = c;
        if (!r.cls) {
            set_error("serve: no multi-limb class for %d words", r.words);
            return MDZGPU_ERR_UNSUPPORTED;
        }
    }
    int rc = half_spacing(&q->span, r.W, &r.hs_m, &r.hs_e);
    if (rc)
        return rc;
    r.julia = q->family == MDZ_FAMILY_JULIA;
    r.tables.assign((size_t)(r.W + r.H + (r.julia ? 2 : 0)) * r.words, 0);
    if (perturb_tables(&q->cx, &q->cy, r.hs_m, r.hs_e, r.W, r.H, r.words, r.tables)) {
        set_error("serve: pixel coordinates must satisfy |x|, |y| < 4");
        return MDZGPU_ERR_RANGE;
    }
    if (r.julia) {
        uint32_t* jw = r.tables.data() + (size_t)(r.W + r.H) * r.words;
        if (fx_from_mpval(&q->julia_re, r.words, jw)
            || fx_from_mpval(&q->julia_im, r.words, jw + r.words)
            || !fx_fits_coordinate(jw, r.words) || !fx_fits_coordinate(jw + r.words, r.words)) {
            set_error("serve: the Julia constant must satisfy |re|, |im| < 4");
            return MDZGPU_ERR_RANGE;
        }
    }
    r.lay = make_layout(r);
    return MDZGPU_OK;
}

// Throughput guesses (pixel-iterations/s on the whole GPU) that turn a step
// duration into per-request budgets.
double class_rate(int cls)
{
    if (cls < kServePerturbClasses)
        return 3.0e11;
    const double w = (double)serve_mp_class_words(cls);
    return 2.0e9 * (34.0 / w) * (34.0 / w);
}

const char* formula_name(int f)
{
    switch (f) {
    case MDZ_MANDELBROT: return "mandelbrot";
    case MDZ_BURNING_SHIP: return "burning_ship";
    case MDZ_GENERALIZED_CELTIC: return "generalized_celtic";
    case MDZ_VARIANT: return "variant";
    default: return "unknown";
    }
}

}  // namespace

struct Server {
    mdzgpu_serve_config cfg{};
    int device = 0, num_sms = 0;
    cudaStream_t main = nullptr;
    cudaStream_t side[kServeSlots] = {};
    // low priority: each request's result copies (fin) and the escalation
    // passes (esc: kEscLanes streams, one request's passes at a time on
    // each), on at most 1 / kEscShare of the SMs together so that the steps
    // keep the rest
    cudaStream_t fin[kServeSlots] = {};
    cudaStream_t esc[kEscLanes] = {};
    // No stream command is ever queued behind a long kernel (it would hold
    // a hardware queue shared with other streams, the steps' among them):
    // the orbit and escalation kernels report their end in pinned host
    // words, and the host queues what follows them.
    std::deque<std::shared_ptr<Req>> esc_fifo;
    std::shared_ptr<Req> esc_cur[kEscLanes];
    char* stage_dev = nullptr;  // device alias of stage_host
    cudaStream_t branch[kServeClasses] = {};
    cudaEvent_t fork = nullptr, join[kServeClasses] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t step_exec = nullptr;
    ServeDev* d = nullptr;
    ServeCtl* ctl_h = nullptr;
    ServeStatus* status_h = nullptr;
    ServeReq* req_h = nullptr;
    unsigned* queues = nullptr;
    char* arena_dev = nullptr;
    char* stage_host = nullptr;
    Arena arena, stage;
    unsigned cur = 0;
    long qhost[kServeClasses] = {};      // entries in queue `cur`
    // budget feedback: each class's slice kernel should take one step;
    // rate_adj scales its throughput guess by the time it actually took
    double rate_adj[kServeClasses];
    double class_ms[kServeClasses] = {};  // summed slice kernel time
    double graph_ms = 0, lead_ms = 0;     // device step spans; begin to first slice
    // per step: host wall time (graph launch to synchronisation) minus the
    // device span of the step (its first to its last kernel)
    std::vector<float> step_gap_ms;
    double loop_ms[9] = {};  // host loop: cancels, admit, orbits, step, finish, idle;
                             // inside step: before the graph, start_finish, graph launch
    long inflight[kServeClasses] = {};   // admitted pixels per class
    std::shared_ptr<Req> slots[kServeSlots];
    int launches_per_step = 0;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Req>> waiting;
    std::unordered_map<int64_t, std::shared_ptr<Req>> all;
    int64_t next_id = 1;
    bool quit = false;
    std::thread th;
    // statistics (guarded by mu)
    mdzgpu_serve_stats st{};
    std::vector<double> latencies;
    FILE* log = nullptr;

    int init(const mdzgpu_serve_config* c);
    void teardown();
    void run();
    int capture_step();
    void admit();
    int setup(const std::shared_ptr<Req>& r);
    void poll_orbits();
    int step();
    int start_finish(const std::shared_ptr<Req>& r);
    int advance_finishing();
    int launch_escalation(const std::shared_ptr<Req>& r, bool mp_pass);
    int enqueue_copies(const std::shared_ptr<Req>& r);
    volatile int* hflag(const std::shared_ptr<Req>& r, int off)
    {
        return (volatile int*)(stage_host + r->host_off + r->lay.h_misc + off);
    }
    volatile int* dflag(const std::shared_ptr<Req>& r, int off)
    {
        return (volatile int*)(stage_dev + r->host_off + r->lay.h_misc + off);
    }
    void poll_finishing();
    void end(const std::shared_ptr<Req>& r, int state, int error);
    void check_cancels();
    int active() const
    {
        int n = 0;
        for (const auto& s : slots)
            n += s != nullptr;
        return n;
    }
};

int Server::init(const mdzgpu_serve_config* c)
{
    if (c)
        cfg = *c;
    if (cfg.max_requests <= 0 || cfg.max_requests > kServeSlots)
        cfg.max_requests = kServeSlots;
    if (cfg.arena_bytes <= 0)
        cfg.arena_bytes = 8LL << 30;
    if (cfg.staging_bytes <= 0)
        cfg.staging_bytes = 512LL << 20;
    if (cfg.queue_pixels <= 0)
        cfg.queue_pixels = 1LL << 23;
    if (cfg.queue_pixels > kServeMaxPixels)
        cfg.queue_pixels = kServeMaxPixels;
    if (cfg.step_ms <= 0)
        cfg.step_ms = 2.0;
    device = cfg.device;
    MDZ_CUDA_TRY(cudaSetDevice(device));
    MDZ_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
    int lo = 0, hi = 0;
    MDZ_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    // priorities: orbits (side) highest, the steps (main) above the result
    // copies and escalation passes (fin, esc), which take what is left
    MDZ_CUDA_TRY(cudaStreamCreateWithPriority(&main, cudaStreamNonBlocking, (lo + hi) / 2));
    for (auto& s : side)
        MDZ_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, hi));
    for (auto& s : fin)
        MDZ_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, lo));
    for (auto& s : esc)
        MDZ_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, lo));
    for (auto& s : branch)
        MDZ_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    MDZ_CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    for (auto& e : join)
        MDZ_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    MDZ_CUDA_TRY(cudaMalloc((void**)&d, sizeof(ServeDev)));
    MDZ_CUDA_TRY(cudaMemset(d, 0, sizeof(ServeDev)));
    {
        ServeStatus s0;
        memset(&s0, 0, sizeof s0);
        for (int c = 0; c < kServeClasses; ++c) {
            s0.tk[0][c][0] = s0.tk[1][c][0] = ~0ull;
            rate_adj[c] = 1.0;
        }
        MDZ_CUDA_TRY(cudaMemcpy(&d->status, &s0, sizeof s0, cudaMemcpyHostToDevice));
    }
    MDZ_CUDA_TRY(cudaHostAlloc((void**)&ctl_h, sizeof(ServeCtl), cudaHostAllocDefault));
    MDZ_CUDA_TRY(cudaHostAlloc((void**)&status_h, sizeof(ServeStatus), cudaHostAllocDefault));
    MDZ_CUDA_TRY(cudaHostAlloc((void**)&req_h, sizeof(ServeReq) * kServeSlots,
                               cudaHostAllocDefault));
    memset(ctl_h, 0, sizeof(ServeCtl));
    memset(status_h, 0, sizeof(ServeStatus));
    memset((void*)req_h, 0, sizeof(ServeReq) * kServeSlots);
    const size_t qbytes = (size_t)cfg.queue_pixels * 4;
    MDZ_CUDA_TRY(cudaMalloc((void**)&queues, qbytes * 2 * kServeClasses));
    {
        unsigned* qptr[kServeClasses][2];
        for (int c = 0; c < kServeClasses; ++c)
            for (int k = 0; k < 2; ++k)
                qptr[c][k] = queues + ((size_t)c * 2 + k) * (size_t)cfg.queue_pixels;
        MDZ_CUDA_TRY(cudaMemcpy(&d->queue[0][0], qptr, sizeof qptr, cudaMemcpyHostToDevice));
    }
    MDZ_CUDA_TRY(cudaMalloc((void**)&arena_dev, (size_t)cfg.arena_bytes));
    MDZ_CUDA_TRY(cudaHostAlloc((void**)&stage_host, (size_t)cfg.staging_bytes,
                               cudaHostAllocMapped));
    MDZ_CUDA_TRY(cudaHostGetDevicePointer((void**)&stage_dev, stage_host, 0));
    arena.reset((size_t)cfg.arena_bytes);
    stage.reset((size_t)cfg.staging_bytes);
    // every kernel the engine may launch is loaded now, while the device
    // is idle; one direct launch of every slice kernel (queues empty: they
    // exit at once) sets their launch attributes outside the capture
    int rc = preload_perturb_kernels();
    if (!rc)
        rc = preload_mp_kernels();
    for (int c = 0; !rc && c < kServePerturbClasses; ++c)
        rc = launch_serve_perturb(d, c, num_sms, main);
    for (int c = kServePerturbClasses; !rc && c < kServeClasses; ++c)
        rc = launch_serve_mp(d, c, num_sms, main);
    if (!rc)
        rc = launch_serve_step_end(d, main);
    if (rc)
        return rc;
    MDZ_CUDA_TRY(cudaStreamSynchronize(main));
    if ((rc = capture_step()))
        return rc;
    if (cfg.log_path && cfg.log_path[0]) {
        log = fopen(cfg.log_path, "a");
        if (!log) {
            set_error("serve: cannot open log %s", cfg.log_path);
            return MDZGPU_ERR_ARG;
        }
    }
    th = std::thread([this] { run(); });
    return MDZGPU_OK;
}

// One step as a graph: control block in, every method's slice kernel in
// parallel branches, queue flip, status out.
int Server::capture_step()
{
    MDZ_CUDA_TRY(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal));
    int rc = MDZGPU_OK;
    launches_per_step = 0;
    if (cudaMemcpyAsync(&d->ctl, ctl_h, sizeof(ServeCtl), cudaMemcpyHostToDevice, main)
        != cudaSuccess)
        rc = MDZGPU_ERR_CUDA;
    if (!rc) {
        rc = launch_serve_step_begin(d, main);
        ++launches_per_step;
    }
    if (!rc && cudaEventRecord(fork, main) != cudaSuccess)
        rc = MDZGPU_ERR_CUDA;
    for (int c = 0; !rc && c < kServeClasses; ++c) {
        if (cudaStreamWaitEvent(branch[c], fork, 0) != cudaSuccess) {
            rc = MDZGPU_ERR_CUDA;
            break;
        }
        rc = c < kServePerturbClasses ? launch_serve_perturb(d, c, num_sms, branch[c])
                                      : launch_serve_mp(d, c, num_sms, branch[c]);
        ++launches_per_step;
        if (!rc && (cudaEventRecord(join[c], branch[c]) != cudaSuccess
                    || cudaStreamWaitEvent(main, join[c], 0) != cudaSuccess))
            rc = MDZGPU_ERR_CUDA;
    }
    if (!rc) {
        rc = launch_serve_step_end(d, main);
        ++launches_per_step;
    }
    if (!rc && cudaMemcpyAsync(status_h, &d->status, sizeof(ServeStatus), cudaMemcpyDeviceToHost,
                               main) != cudaSuccess)
        rc = MDZGPU_ERR_CUDA;
    const cudaError_t e = cudaStreamEndCapture(main, &graph);
    if (rc) {
        set_error("serve: step capture failed");
        return rc;
    }
    MDZ_CUDA_TRY(e);
    MDZ_CUDA_TRY(cudaGraphInstantiate(&step_exec, graph, 0));
    return MDZGPU_OK;
}

void Server::end(const std::shared_ptr<Req>& r, int state, int error)
{
    if (r->slot >= 0) {
        arena.release(r->dev_off, r->lay.dev_bytes);
        stage.release(r->host_off, r->lay.host_bytes);
        inflight[r->cls] -= (long)r->npix;
        slots[r->slot] = nullptr;
        r->slot = -1;
    }
    if (r->ev_done)
        cudaEventDestroy(r->ev_done);
    r->ev_done = nullptr;
    r->phase = kEnded;
    std::lock_guard<std::mutex> lk(mu);
    r->state = state;
    r->error = error;
    r->t_done = wall_ms();
    if (state == MDZGPU_REQ_DONE) {
        st.completed++;
        st.pixel_iters += r->pixel_iters;
        latencies.push_back(r->t_done - r->t_submit);
        if (log) {
            const double lat = r->t_done - r->t_submit;
            fprintf(log,
                    "{\"id\": %lld, \"width\": %d, \"height\": %d, \"precision\": %ld, "
                    "\"formula\": \"%s\", \"depth\": %u, \"method\": \"%s\", \"words\": %d, "
                    "\"pixel_iters\": %lld, \"queue_ms\": %.3f, \"latency_ms\": %.3f, "
                    "\"pixel_iters_per_s\": %.6g, \"escalated_fp64\": %lld, "
                    "\"escalated_mp\": %lld, \"steps\": %lld, \"main_ms\": %.3f, "
                    "\"esc_wait_ms\": %.3f, \"esc_ms\": %.3f}\n",
                    (long long)r->id, r->W, r->H, r->precision, formula_name(r->fractal),
                    r->depth, r->method == MDZGPU_METHOD_PERTURB ? "perturbation" : "multi_limb",
                    r->method == MDZGPU_METHOD_PERTURB ? r->limbs : r->words,
                    (long long)r->pixel_iters, r->t_admit - r->t_submit, lat,
                    lat > 0 ? (double)r->pixel_iters / (lat * 1e-3) : 0.0,
                    (long long)r->esc_fp64, (long long)r->esc_mp, (long long)r->steps,
                    r->t_main > 0 ? r->t_main - r->t_submit : 0.0,
                    r->t_esc0 > 0 ? r->t_esc0 - r->t_main : 0.0,
                    r->t_esc1 > 0 ? r->t_esc1 - r->t_esc0 : 0.0);
            fflush(log);
        }
    } else if (state == MDZGPU_REQ_FAILED) {
        st.failed++;
    } else if (state == MDZGPU_REQ_TIMEOUT) {
        st.timed_out++;
    } else {
        st.cancelled++;
    }
    cv_done.notify_all();
}

void Server::check_cancels()
{
    const double now = wall_ms();
    std::vector<std::shared_ptr<Req>> drop;
    {
        std::lock_guard<std::mutex> lk(mu);
        for (auto it = waiting.begin(); it != waiting.end();) {
            auto& r = *it;
            if (!r->cancel && r->timeout_ms > 0 && now - r->t_submit > r->timeout_ms) {
                r->cancel = true;
                r->cancel_state = MDZGPU_REQ_TIMEOUT;
            }
            if (r->cancel) {
                drop.push_back(r);
                it = waiting.erase(it);
            } else {
                ++it;
            }
        }
        for (auto& s : slots)
            if (s && !s->cancel && s->timeout_ms > 0 && now - s->t_submit > s->timeout_ms
                && s->phase == kRunning) {
                s->cancel = true;
                s->cancel_state = MDZGPU_REQ_TIMEOUT;
            }
    }
    for (auto& r : drop)
        end(r, r->cancel_state, 0);
}

void Server::admit()
{
    for (;;) {
        std::shared_ptr<Req> r;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (waiting.empty())
                return;
            r = waiting.front();
        }
        int slot = -1;
        for (int s = 0; s < cfg.max_requests; ++s)
            if (!slots[s]) {
                slot = s;
                break;
            }
        if (slot < 0 || inflight[r->cls] + (long)r->npix > cfg.queue_pixels)
            return;
        size_t doff = 0, hoff = 0;
        if (!arena.alloc(r->lay.dev_bytes, &doff))
            return;
        if (!stage.alloc(r->lay.host_bytes, &hoff)) {
            arena.release(doff, r->lay.dev_bytes);
            return;
        }
        r->dev_off = doff;
        r->host_off = hoff;
        r->slot = slot;
        slots[slot] = r;
        inflight[r->cls] += (long)r->npix;
        {
            std::lock_guard<std::mutex> lk(mu);
            waiting.pop_front();
            r->state = MDZGPU_REQ_RUNNING;
            r->t_admit = wall_ms();
            const int64_t used = (int64_t)arena.used();
            st.device_bytes_in_use = used;
            st.device_bytes_peak = std::max(st.device_bytes_peak, used);
        }
        const int rc = setup(r);
        if (rc)
            end(r, MDZGPU_REQ_FAILED, rc);
    }
}

int Server::setup(const std::shared_ptr<Req>& r)
{
    const Layout& l = r->lay;
    char* db = arena_dev + r->dev_off;
    char* hb = stage_host + r->host_off;
    memcpy(hb + l.h_tables, r->tables.data(), r->tables.size() * 4);
    MDZ_CUDA_TRY(cudaMemcpyAsync(db + l.tables, hb + l.h_tables, r->tables.size() * 4,
                                 cudaMemcpyHostToDevice, main));
    MDZ_CUDA_TRY(cudaMemsetAsync(db + l.sync, 0, 256, main));
    ServeReq& q = req_h[r->slot];
    memset((void*)&q, 0, sizeof q);
    PerturbLaunch& p = q.pl;
    p = PerturbLaunch{};
    p.W = r->W;
    p.H = r->H;
    p.row0 = 0;
    p.nrows = r->H;
    p.depth = r->depth;
    p.hs_m = r->hs_m;
    p.hs_e = r->hs_e;
    p.out = (int32_t*)(db + l.counts);
    p.mag = r->want_mag ? (float*)(db + l.mag) : nullptr;
    p.sync = (FrameSync*)(db + l.sync);
    q.xs = (const uint32_t*)(db + l.tables);
    q.ys = q.xs + (size_t)r->W * r->words;
    q.julia = r->julia ? q.xs + (size_t)(r->W + r->H) * r->words : nullptr;
    q.fractal = r->fractal;
    q.words = r->words;
    q.state = (uint4*)(db + l.state);
    if (r->method == MDZGPU_METHOD_PERTURB) {
        char* ob = db + l.orbit;
        const OrbitLayout& ol = l.ol;
        memcpy(hb + l.h_digits, r->digits.data(), r->digits.size() * 4);
        MDZ_CUDA_TRY(cudaMemcpyAsync(ob + ol.dig, hb + l.h_digits, r->digits.size() * 4,
                                     cudaMemcpyHostToDevice, main));
        MDZ_CUDA_TRY(cudaMemsetAsync(ob + ol.len, 0, 256, main));
        MDZ_CUDA_TRY(cudaMemsetAsync(ob + ol.reb, 0, 256, main));
        MDZ_CUDA_TRY(cudaMemsetAsync(db + l.lists, 0, 256, main));
        p.zq = (const float4*)ob;
        p.zd = (const double2*)(ob + ol.zd);
        p.ze = (const int*)(ob + ol.ze);
        p.dd = (const double*)(ob + ol.dd);
        p.de = (const int*)(ob + ol.de);
        p.orbit_len = (const int*)(ob + ol.len);
        p.tiny = (const unsigned*)(ob + ol.tiny);
        p.att = (const unsigned*)(ob + ol.att);
        p.fractal = r->fractal;
        p.fm = (const double*)(ob + ol.fm);
        p.fe = (const int*)(ob + ol.fe);
        p.axis = (const unsigned*)(ob + ol.axis);
        p.rebases = (unsigned long long*)(ob + ol.reb);
        p.lost_limit = 1.0f;  // bits a pixel may lose before its FP64 re-run
        p.flag_out = (unsigned*)(db + l.lists + 256);
        p.flag_out_count = (unsigned*)(db + l.lists);
        // progress of the streamed orbit (beside out_len, zeroed above)
        int* prog = (int*)(ob + ol.len);
        p.raw_len = prog + 1;
        p.fin_len = prog + 2;
        p.orbit_done = prog + 3;
        p.orbit_error = prog + 4;
        q.state_stride = 2;
        MDZ_CUDA_TRY(cudaMemcpyAsync(&d->req[r->slot], &q, sizeof q, cudaMemcpyHostToDevice,
                                     main));
        OrbitLaunch o;
        o.limbs = r->limbs;
        o.c_re = (const int*)(ob + ol.dig);
        o.c_im = o.c_re + r->limbs;
        o.zq = (float4*)ob;
        o.zd = (double2*)(ob + ol.zd);
        o.ze = (int*)(ob + ol.ze);
        o.dd = (double*)(ob + ol.dd);
        o.de = (int*)(ob + ol.de);
        o.digits = (int*)(ob + ol.raw);
        o.max_k = (int)r->depth + 1;
        o.out_len = (int*)(ob + ol.len);
        o.tiny = (unsigned*)(ob + ol.tiny);
        o.att = (unsigned*)(ob + ol.att);
        o.fractal = r->fractal;
        o.fm = (double*)(ob + ol.fm);
        o.fe = (int*)(ob + ol.fe);
        o.axis = (unsigned*)(ob + ol.axis);
        o.sm_busy = d->sm_busy;
        o.sm_words = kServeSmWords;
        cudaEvent_t ready;
        MDZ_CUDA_TRY(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
        cudaEventRecord(ready, main);
        cudaStreamWaitEvent(side[r->slot], ready, 0);
        cudaEventDestroy(ready);
        // the orbit streams: pixels join the queue now and iterate up to
        // the last finished entry at every step; its end (1, or 2 when the
        // finisher gave up) lands in the host word h_misc + 16
        *hflag(r, 16) = 0;
        int rc = launch_orbit_stream(o, prog, side[r->slot],
                                     DoneSignal{(unsigned*)(prog + 6), dflag(r, 16)});
        if (rc)
            return rc;
        rc = launch_serve_enqueue(d, r->cls, (int)cur, r->slot, (unsigned)r->npix, main);
        if (rc)
            return rc;
        qhost[r->cls] += (long)r->npix;
        r->orbit_running = true;
        r->phase = kRunning;
        std::lock_guard<std::mutex> lk(mu);
        st.launches += 3;
    } else {
        q.state_stride = serve_mp_state_stride(r->words);
        MDZ_CUDA_TRY(cudaMemcpyAsync(&d->req[r->slot], &q, sizeof q, cudaMemcpyHostToDevice,
                                     main));
        int rc = launch_serve_enqueue(d, r->cls, (int)cur, r->slot, (unsigned)r->npix, main);
        if (rc)
            return rc;
        qhost[r->cls] += (long)r->npix;
        r->phase = kRunning;
        std::lock_guard<std::mutex> lk(mu);
        st.launches += 2;
    }
    return MDZGPU_OK;
}

void Server::poll_orbits()
{
    for (auto& r : slots) {
        if (!r || !r->orbit_running)
            continue;
        const int v = *hflag(r, 16);
        if (v == 0)
            continue;
        r->orbit_running = false;
        const int err = v != 1;
        if (err) {
            // the finisher gave up (or the launch failed): its pixels can not
            // finish; drop them and fail the request
            set_error("serve: reference orbit of request %lld failed", (long long)r->id);
            std::lock_guard<std::mutex> lk(mu);
            r->cancel = true;
            r->cancel_state = MDZGPU_REQ_FAILED;
        }
    }
}

int Server::step()
{
    const double t_pre = wall_ms();
    // budgets: each running request gets an equal share of the step
    int R = 0;
    for (auto& r : slots)
        R += r && r->phase == kRunning;
    memset(ctl_h, 0, sizeof(ServeCtl));
    ctl_h->cur = cur;
    bool steered[kServeClasses] = {};  // a budget of the class is above its floor
    {
        std::lock_guard<std::mutex> lk(mu);
        for (int s = 0; s < kServeSlots; ++s) {
            const auto& r = slots[s];
            if (!r || r->phase != kRunning)
                continue;
            if (r->cancel)
                ctl_h->cancel |= 1ull << s;
            unsigned left = status_h->remaining[s];
            if (left == 0 || left > r->npix)
                left = (unsigned)r->npix;  // enqueued since the last status
            const double b =
                cfg.step_ms * 1e-3 * class_rate(r->cls) * rate_adj[r->cls] / ((double)R * left);
            const double bmin = r->cls == 0 ? 256.0 : 16.0;
            ctl_h->budget[s] = (unsigned)std::min(std::max(b, bmin), (double)(1u << 24));
            steered[r->cls] = steered[r->cls] || b > bmin;
        }
    }
    bool had[kServeClasses];
    for (int c = 0; c < kServeClasses; ++c)
        had[c] = qhost[c] > 0;
    const double t0 = wall_ms();
    loop_ms[6] += t0 - t_pre;
    MDZ_CUDA_TRY(cudaGraphLaunch(step_exec, main));
    loop_ms[8] += wall_ms() - t0;
    MDZ_CUDA_TRY(cudaStreamSynchronize(main));
    const double t1 = wall_ms();
    {
        const unsigned long long b0 = status_h->tstep[cur][0], b1 = status_h->tstep[cur][1];
        unsigned long long first = ~0ull;
        for (int c = 0; c < kServeClasses; ++c)
            if (had[c])
                first = std::min(first, status_h->tk[cur][c][0]);
        if (b1 > b0) {
            graph_ms += (double)(b1 - b0) * 1e-6;
            if (step_gap_ms.size() < (1u << 20))
                step_gap_ms.push_back((float)(t1 - t0 - (double)(b1 - b0) * 1e-6));
            if (first != ~0ull && first > b0)
                lead_ms += (double)(first - b0) * 1e-6;
        }
    }
    for (int c = 0; c < kServeClasses; ++c) {
        const unsigned long long a = status_h->tk[cur][c][0], b = status_h->tk[cur][c][1];
        if (!had[c] || a == ~0ull || b <= a)
            continue;
        const double ms = (double)(b - a) * 1e-6;
        class_ms[c] += ms;
        // fast down, slow up; the guess stays within [1e-4, 4] of itself
        const double ratio = cfg.step_ms / std::max(ms, 1e-3);
        const double f = ratio < 1.0 ? std::max(ratio, 0.25) : pow(std::min(ratio, 4.0), 0.25);
        if (ratio < 1.0 && !steered[c])
            continue;  // every budget at its floor: the time is not the budgets'
        rate_adj[c] = std::min(std::max(rate_adj[c] * f, 1e-4), 4.0);
    }
    cur ^= 1u;
    for (int c = 0; c < kServeClasses; ++c)
        qhost[c] = (long)status_h->qcount[c][cur];
    {
        std::lock_guard<std::mutex> lk(mu);
        st.steps++;
        st.launches += launches_per_step;
        st.busy_ms += t1 - t0;
    }
    for (int s = 0; s < kServeSlots; ++s) {
        auto r = slots[s];
        if (!r || r->phase != kRunning)
            continue;
        {
            std::lock_guard<std::mutex> lk(mu);
            r->steps++;
        }
        if (status_h->remaining[s] != 0) {
            if (qhost[r->cls] == 0) {
                // pixels neither finished nor queued: never expected; fail the
                // request rather than wait for it forever
                set_error("serve: request %lld lost %u pixels", (long long)r->id,
                          status_h->remaining[s]);
                end(r, MDZGPU_REQ_FAILED, MDZGPU_ERR_CUDA);
            }
            continue;
        }
        bool cancel;
        {
            std::lock_guard<std::mutex> lk(mu);
            cancel = r->cancel;
        }
        if (cancel) {
            // the orbit may still run: the memory is released once it ends
            r->cancelled = true;
            r->phase = kCopyWait;
            continue;
        }
        const double tf = wall_ms();
        const int rc = start_finish(r);
        loop_ms[7] += wall_ms() - tf;
        if (rc)
            end(r, MDZGPU_REQ_FAILED, rc);
    }
    return MDZGPU_OK;
}

// Main pass done.  A perturbation request whose FP32 pass flagged pixels
// queues for the escalation passes (FP64, then multi-limb over what FP64
// could not settle), which run on kEscLanes low-priority streams, one
// request at a time on each, with 1 / kEscShare of the SMs between them, so
// that a request with many flagged pixels delays its own result, not the
// steps of the others (nor, with a second lane, every escalation behind
// it).
// Every other request waits only for its orbit launch to end (the arena is
// released only once nothing writes it), then copies its results out.
int Server::start_finish(const std::shared_ptr<Req>& r)
{
    // the step that finished the FP32 pass reported how many it flagged
    const unsigned flagged = r->method == MDZGPU_METHOD_PERTURB ? status_h->flagged[r->slot] : 0u;
    r->flagged = flagged;
    r->t_main = wall_ms();
    if (flagged != 0) {
        esc_fifo.push_back(r);
        r->phase = kEscWait;
    } else {
        memset(stage_host + r->host_off + r->lay.h_misc, 0, 8);  // no escalation
        r->phase = kCopyWait;
    }
    return MDZGPU_OK;
}

// One chunk of an escalation pass: list tiles esc_base + [0, chunk), on
// 1 / kEscShare of the SMs while other requests run, on all of them when
// the passes are the only work left.
int Server::launch_escalation(const std::shared_ptr<Req>& r, bool mp_pass)
{
    const Layout& l = r->lay;
    char* db = arena_dev + r->dev_off;
    bool alone;
    {
        std::lock_guard<std::mutex> lk(mu);
        alone = waiting.empty();
    }
    for (const auto& o : slots)
        alone = alone && (!o || o->phase > kRunning);
    int lanes = 0;
    for (const auto& e : esc_cur)
        lanes += e ? 1 : 0;
    mdzgpu_ctx shape;  // the list passes read only the SM count
    shape.device = device;
    shape.num_sms = std::max(1, (alone ? num_sms : num_sms / kEscShare) / std::max(1, lanes));
    const unsigned chunk = (unsigned)shape.num_sms * kEscTilesPerSm;
    PerturbLaunch p = req_h[r->slot].pl;
    unsigned* counts_dev = (unsigned*)(db + l.lists);
    unsigned* list1 = (unsigned*)(db + l.lists + 256);
    unsigned* list2 = list1 + r->npix;
    // the sync block (tile counter, exit count at +128) starts at zero
    cudaStream_t es = esc[r->esc_lane];
    MDZ_CUDA_TRY(cudaMemsetAsync(db + l.sync, 0, 256, es));
    const DoneSignal done{(unsigned*)(db + l.sync + 128), dflag(r, mp_pass ? 24 : 20)};
    *hflag(r, mp_pass ? 24 : 20) = 0;
    int rc;
    if (!mp_pass) {
        p.list_in = list1;
        p.list_in_count = counts_dev;
        p.lost_limit = 6.0f;  // FP64 pass: bits before the multi-limb re-run
        p.flag_out = list2;
        p.flag_out_count = counts_dev + 1;
        p.done = done;
        p.tile_base = r->esc_base;
        p.tile_limit = chunk;
        rc = launch_perturb(&shape, p, es, 1);
    } else {
        MpLaunch q;
        q.W = r->W;
        q.H = r->H;
        q.row0 = 0;
        q.nrows = r->H;
        q.family = MDZ_FAMILY_MANDEL;
        q.fractal = r->fractal;
        q.depth = r->depth;
        q.words = r->words;
        q.xs = (const uint32_t*)(db + l.tables);
        q.ys = q.xs + (size_t)r->W * r->words;
        q.julia = q.xs;
        q.out = p.out;
        q.sync = (FrameSync*)(db + l.sync);
        q.tile_rows_done = nullptr;
        q.band_flags = nullptr;
        q.stop = nullptr;
        q.list = list2;
        q.list_count = counts_dev + 1;
        q.mag = p.mag;
        q.done = done;
        q.tile_base = r->esc_base;
        q.tile_limit = chunk;
        rc = launch_mp(&shape, q, es);
    }
    r->esc_base += chunk;
    if (!rc) {
        std::lock_guard<std::mutex> lk(mu);
        st.launches += 1;
    }
    return rc;
}

// Copies out on the request's fin stream (nothing long runs before them).
int Server::enqueue_copies(const std::shared_ptr<Req>& r)
{
    const Layout& l = r->lay;
    char* db = arena_dev + r->dev_off;
    char* hb = stage_host + r->host_off;
    cudaStream_t s = fin[r->slot];
    if (r->method == MDZGPU_METHOD_PERTURB) {
        if (r->phase == kEscMp)  // escalated: the lists' counts
            MDZ_CUDA_TRY(cudaMemcpyAsync(hb + l.h_misc, db + l.lists, 8, cudaMemcpyDeviceToHost,
                                         s));
        MDZ_CUDA_TRY(cudaMemcpyAsync(hb + l.h_misc + 8, db + l.orbit + l.ol.reb, 8,
                                     cudaMemcpyDeviceToHost, s));
    }
    MDZ_CUDA_TRY(cudaMemcpyAsync(hb + l.h_counts, db + l.counts, r->npix * 4,
                                 cudaMemcpyDeviceToHost, s));
    if (r->want_mag)
        MDZ_CUDA_TRY(cudaMemcpyAsync(hb + l.h_mag, db + l.mag, r->npix * 4,
                                     cudaMemcpyDeviceToHost, s));
    MDZ_CUDA_TRY(cudaEventCreateWithFlags(&r->ev_done, cudaEventDisableTiming));
    MDZ_CUDA_TRY(cudaEventRecord(r->ev_done, s));
    r->phase = kFinishing;
    return MDZGPU_OK;
}

int Server::advance_finishing()
{
    // a cancel after the main pass: no further passes, no copies to the
    // caller (a pass in flight ends first; copies already queued land in
    // staging only)
    for (auto& slot_ref : slots) {
        auto r = slot_ref;
        if (!r || r->phase <= kRunning || r->cancelled)
            continue;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (!r->cancel)
                continue;
        }
        r->cancelled = true;
        if (r->phase == kEscWait) {
            for (auto it = esc_fifo.begin(); it != esc_fifo.end(); ++it)
                if (*it == r) {
                    esc_fifo.erase(it);
                    break;
                }
            r->phase = kCopyWait;
        }
    }
    // results of requests whose kernels have all ended
    for (auto& slot_ref : slots) {
        auto r = slot_ref;
        if (!r || r->phase != kCopyWait || r->orbit_running)
            continue;
        if (r->cancelled) {
            end(r, r->cancel_state, 0);
            continue;
        }
        if (int rc = enqueue_copies(r))
            end(r, MDZGPU_REQ_FAILED, rc);
    }
    // the escalation chunks in flight: 1 = more of the list is left, 3 = the
    // pass reached the list's end
    for (int k = 0; k < kEscLanes; ++k) {
        if (!esc_cur[k])
            continue;
        auto r = esc_cur[k];
        const int v = *hflag(r, r->phase == kEscFp64 ? 20 : 24);
        int rc = MDZGPU_OK;
        if (v != 0 && r->cancelled) {
            esc_cur[k] = nullptr;   // cancelled: its memory goes once the orbit ended
            r->phase = kCopyWait;
        } else if (v == 1) {
            rc = launch_escalation(r, r->phase == kEscMp);
        } else if (v == 3 && r->phase == kEscFp64) {
            r->phase = kEscMp;
            r->esc_base = 0;
            rc = launch_escalation(r, true);
        } else if (v == 3) {
            esc_cur[k] = nullptr;
            r->t_esc1 = wall_ms();
            rc = enqueue_copies(r);
        }
        if (rc) {
            esc_cur[k] = nullptr;
            end(r, MDZGPU_REQ_FAILED, rc);
        }
    }
    // free lanes take the least work (flagged pixels x depth) among those
    // whose orbit ended
    for (int k = 0; k < kEscLanes; ++k) {
        if (esc_cur[k])
            continue;
        auto best = esc_fifo.end();
        for (auto it = esc_fifo.begin(); it != esc_fifo.end(); ++it) {
            if ((*it)->orbit_running)
                continue;
            if (best == esc_fifo.end()
                || (double)(*it)->flagged * (*it)->depth < (double)(*best)->flagged * (*best)->depth)
                best = it;
        }
        if (best == esc_fifo.end())
            break;
        auto r = *best;
        esc_fifo.erase(best);
        esc_cur[k] = r;
        r->esc_lane = k;
        r->phase = kEscFp64;
        r->esc_base = 0;
        r->t_esc0 = wall_ms();
        if (int rc = launch_escalation(r, false)) {
            esc_cur[k] = nullptr;
            end(r, MDZGPU_REQ_FAILED, rc);
        }
    }
    return MDZGPU_OK;
}

void Server::poll_finishing()
{
    for (auto& slot_ref : slots) {
        auto r = slot_ref;
        if (!r || r->phase != kFinishing)
            continue;
        const cudaError_t e = cudaEventQuery(r->ev_done);
        if (e == cudaErrorNotReady)
            continue;
        if (e != cudaSuccess) {
            set_error("serve: request %lld failed: %s", (long long)r->id, cudaGetErrorString(e));
            end(r, MDZGPU_REQ_FAILED, MDZGPU_ERR_CUDA);
            continue;
        }
        if (r->cancelled) {
            end(r, r->cancel_state, 0);
            continue;
        }
        const Layout& l = r->lay;
        const char* hb = stage_host + r->host_off;
        const int32_t* c = (const int32_t*)(hb + l.h_counts);
        memcpy(r->out_counts, c, r->npix * 4);
        if (r->want_mag)
            memcpy(r->out_mag, hb + l.h_mag, r->npix * 4);
        int64_t its = 0;
        for (size_t i = 0; i < r->npix; ++i)
            its += c[i] ? c[i] : (int64_t)r->depth;
        r->pixel_iters = its;
        if (r->method == MDZGPU_METHOD_PERTURB) {
            const unsigned* esc = (const unsigned*)(hb + l.h_misc);
            r->esc_fp64 = esc[0];
            r->esc_mp = esc[1];
            unsigned long long reb;
            memcpy(&reb, hb + l.h_misc + 8, 8);
            r->rebases = (int64_t)reb;
        }
        end(r, MDZGPU_REQ_DONE, 0);
    }
}

void Server::run()
{
    cudaSetDevice(device);
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(mu);
            if (quit)
                break;
            bool idle = waiting.empty();
            for (const auto& s : slots)
                idle = idle && !s;
            if (idle)
                cv_work.wait_for(lk, std::chrono::milliseconds(20));
            if (quit)
                break;
        }
        double ta = wall_ms();
        check_cancels();
        double tb = wall_ms();
        loop_ms[0] += tb - ta;
        admit();
        ta = wall_ms();
        loop_ms[1] += ta - tb;
        poll_orbits();
        tb = wall_ms();
        loop_ms[2] += tb - ta;
        long queued = 0;
        for (long q : qhost)
            queued += q;
        if (queued > 0) {
            const int step_rc = step();
            ta = wall_ms();
            loop_ms[3] += ta - tb;
            tb = ta;
            if (step_rc) {
                // a failed step leaves the device state unknown: fail everything
                for (int k = 0; k < kEscLanes; ++k) {
                    cudaStreamSynchronize(esc[k]);
                    esc_cur[k] = nullptr;
                }
                esc_fifo.clear();
                for (auto& s : slots)
                    if (s) {
                        auto keep = s;
                        cudaStreamSynchronize(side[keep->slot]);
                        cudaStreamSynchronize(fin[keep->slot]);
                        end(keep, MDZGPU_REQ_FAILED, MDZGPU_ERR_CUDA);
                    }
                for (long& q : qhost)
                    q = 0;
            }
        }
        advance_finishing();
        poll_finishing();
        ta = wall_ms();
        loop_ms[4] += ta - tb;
        if (queued == 0) {
            bool waiting_gpu = false;
            for (const auto& s : slots)
                waiting_gpu = waiting_gpu || (s && (s->orbit_running || s->phase > kRunning));
            if (waiting_gpu)
                std::this_thread::sleep_for(std::chrono::microseconds(100));
            loop_ms[5] += wall_ms() - ta;
        }
    }
    // shutdown: let the GPU work in flight end, then cancel what is left
    cudaStreamSynchronize(main);
    for (auto& s : side)
        cudaStreamSynchronize(s);
    for (auto& s : fin)
        cudaStreamSynchronize(s);
    for (int k = 0; k < kEscLanes; ++k) {
        cudaStreamSynchronize(esc[k]);
        esc_cur[k] = nullptr;
    }
    esc_fifo.clear();
    for (auto& s : slots)
        if (s) {
            auto keep = s;
            end(keep, MDZGPU_REQ_CANCELLED, 0);
        }
    std::deque<std::shared_ptr<Req>> left;
    {
        std::lock_guard<std::mutex> lk(mu);
        left.swap(waiting);
    }
    for (auto& r : left)
        end(r, MDZGPU_REQ_CANCELLED, 0);
}

void Server::teardown()
{
    if (th.joinable()) {
        {
            std::lock_guard<std::mutex> lk(mu);
            quit = true;
        }
        cv_work.notify_all();
        th.join();
    }
    if (main)
        cudaStreamSynchronize(main);
    if (step_exec)
        cudaGraphExecDestroy(step_exec);
    if (graph)
        cudaGraphDestroy(graph);
    for (auto& e : join)
        if (e)
            cudaEventDestroy(e);
    if (fork)
        cudaEventDestroy(fork);
    for (auto& s : branch)
        if (s)
            cudaStreamDestroy(s);
    for (auto& s : side)
        if (s)
            cudaStreamDestroy(s);
    for (auto& s : fin)
        if (s)
            cudaStreamDestroy(s);
    for (auto& s : esc)
        if (s)
            cudaStreamDestroy(s);
    if (main)
        cudaStreamDestroy(main);
    cudaFree(arena_dev);
    cudaFree(queues);
    cudaFree(d);
    cudaFreeHost(stage_host);
    cudaFreeHost(ctl_h);
    cudaFreeHost(status_h);
    cudaFreeHost(req_h);
    if (log) {
        fprintf(log,
                "{\"loop_ms\": {\"cancels\": %.1f, \"admit\": %.1f, \"orbits\": %.1f, "
                "\"step\": %.1f, \"finish\": %.1f, \"idle\": %.1f, \"step_pre_graph\": %.1f, "
                "\"step_start_finish\": %.1f, \"graph_launch\": %.1f}, ",
                loop_ms[0], loop_ms[1], loop_ms[2], loop_ms[3], loop_ms[4], loop_ms[5],
                loop_ms[6], loop_ms[7], loop_ms[8]);
        fprintf(log, "\"device_step_ms\": %.3f, \"step_lead_ms\": %.3f, ", graph_ms, lead_ms);
        if (!step_gap_ms.empty()) {
            std::vector<float> g = step_gap_ms;
            std::sort(g.begin(), g.end());
            auto q = [&](double f) { return g[(size_t)(f * (double)(g.size() - 1))]; };
            fprintf(log, "\"step_gap_ms\": {\"n\": %zu, \"min\": %.4f, \"p10\": %.4f, "
                    "\"p50\": %.4f, \"p90\": %.4f}, ", g.size(), q(0.0), q(0.1), q(0.5), q(0.9));
        }
        fprintf(log, "\"slice_kernel_ms\": [");
        for (int c = 0; c < kServeClasses; ++c)
            fprintf(log, "%s%.3f", c ? ", " : "", class_ms[c]);
        fprintf(log, "], \"rate_adjust\": [");
        for (int c = 0; c < kServeClasses; ++c)
            fprintf(log, "%s%.4g", c ? ", " : "", rate_adj[c]);
        fprintf(log, "]}\n");
        fclose(log);
    }
}

}  // namespace mdz

using namespace mdz;

struct mdzgpu_server {
    Server s;
};

extern "C" {

mdzgpu_server* mdzgpu_serve_create(const mdzgpu_serve_config* cfg)
{
    auto* srv = new mdzgpu_server();
    if (srv->s.init(cfg)) {
        srv->s.teardown();
        delete srv;
        return nullptr;
    }
    return srv;
}

void mdzgpu_serve_destroy(mdzgpu_server* srv)
{
    if (!srv)
        return;
    srv->s.teardown();
    delete srv;
}

int mdzgpu_serve_footprint(const mdzgpu_request* q, int64_t* device_bytes, int64_t* host_bytes)
{
    Req r;
    const int rc = prepare(q, r);
    if (rc)
        return rc;
    if (device_bytes)
        *device_bytes = (int64_t)r.lay.dev_bytes;
    if (host_bytes)
        *host_bytes = (int64_t)r.lay.host_bytes;
    return MDZGPU_OK;
}

int mdzgpu_serve_submit(mdzgpu_server* srv, const mdzgpu_request* q, int64_t* id)
{
    if (!srv) {
        set_error("serve: null server");
        return MDZGPU_ERR_ARG;
    }
    Server& s = srv->s;
    auto r = std::make_shared<Req>();
    int rc = prepare(q, *r);
    if (rc) {
        std::lock_guard<std::mutex> lk(s.mu);
        s.st.submitted++;
        s.st.failed++;
        return rc;
    }
    if (r->lay.dev_bytes > s.arena.size() || r->lay.host_bytes > s.stage.size()
        || (long)r->npix > s.cfg.queue_pixels) {
        set_error("serve: request needs %zu device / %zu host bytes; the server has %lld / %lld",
                  r->lay.dev_bytes, r->lay.host_bytes, (long long)s.cfg.arena_bytes,
                  (long long)s.cfg.staging_bytes);
        std::lock_guard<std::mutex> lk(s.mu);
        s.st.submitted++;
        s.st.failed++;
        return MDZGPU_ERR_NOMEM;
    }
    {
        std::lock_guard<std::mutex> lk(s.mu);
        if (s.quit) {
            set_error("serve: server is stopping");
            return MDZGPU_ERR_STOPPED;
        }
        r->id = s.next_id++;
        r->t_submit = wall_ms();
        s.all[r->id] = r;
        s.waiting.push_back(r);
        s.st.submitted++;
    }
    s.cv_work.notify_all();
    if (id)
        *id = r->id;
    return MDZGPU_OK;
}

static void fill_status(const Req& r, mdzgpu_request_status* out)
{
    memset(out, 0, sizeof *out);
    out->state = r.state;
    out->error = r.error;
    out->method = r.method;
    out->words = r.method == MDZGPU_METHOD_PERTURB ? r.limbs : r.words;
    out->queue_ms = r.t_admit > 0 ? r.t_admit - r.t_submit : 0.0;
    out->latency_ms = r.t_done > 0 ? r.t_done - r.t_submit : 0.0;
    out->pixel_iters = r.pixel_iters;
    out->escalated_fp64 = r.esc_fp64;
    out->escalated_mp = r.esc_mp;
    out->rebases = r.rebases;
    out->steps = r.steps;
    out->main_ms = r.t_main > 0 ? r.t_main - r.t_submit : 0.0;
    out->esc_wait_ms = r.t_esc0 > 0 ? r.t_esc0 - r.t_main : 0.0;
    out->esc_ms = r.t_esc1 > 0 ? r.t_esc1 - r.t_esc0 : 0.0;
}

int mdzgpu_serve_poll(mdzgpu_server* srv, int64_t id, mdzgpu_request_status* out)
{
    if (!srv || !out) {
        set_error("serve: null argument");
        return MDZGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(srv->s.mu);
    auto it = srv->s.all.find(id);
    if (it == srv->s.all.end()) {
        set_error("serve: unknown request %lld", (long long)id);
        return MDZGPU_ERR_ARG;
    }
    fill_status(*it->second, out);
    return MDZGPU_OK;
}

int mdzgpu_serve_wait(mdzgpu_server* srv, int64_t id, double timeout_ms,
                      mdzgpu_request_status* out)
{
    if (!srv) {
        set_error("serve: null server");
        return MDZGPU_ERR_ARG;
    }
    Server& s = srv->s;
    std::unique_lock<std::mutex> lk(s.mu);
    auto it = s.all.find(id);
    if (it == s.all.end()) {
        set_error("serve: unknown request %lld", (long long)id);
        return MDZGPU_ERR_ARG;
    }
    auto r = it->second;
    auto finished = [&] {
        return r->state != MDZGPU_REQ_QUEUED && r->state != MDZGPU_REQ_RUNNING;
    };
    if (timeout_ms < 0)
        s.cv_done.wait(lk, finished);
    else
        s.cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), finished);
    if (out)
        fill_status(*r, out);
    if (!finished()) {
        set_error("serve: request %lld still running", (long long)id);
        return MDZGPU_ERR_TIMEOUT;
    }
    return MDZGPU_OK;
}

int mdzgpu_serve_cancel(mdzgpu_server* srv, int64_t id)
{
    if (!srv) {
        set_error("serve: null server");
        return MDZGPU_ERR_ARG;
    }
    {
        std::lock_guard<std::mutex> lk(srv->s.mu);
        auto it = srv->s.all.find(id);
        if (it == srv->s.all.end()) {
            set_error("serve: unknown request %lld", (long long)id);
            return MDZGPU_ERR_ARG;
        }
        it->second->cancel = true;
        it->second->cancel_state = MDZGPU_REQ_CANCELLED;
    }
    srv->s.cv_work.notify_all();
    return MDZGPU_OK;
}

int mdzgpu_serve_release(mdzgpu_server* srv, int64_t id)
{
    if (!srv) {
        set_error("serve: null server");
        return MDZGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(srv->s.mu);
    auto it = srv->s.all.find(id);
    if (it == srv->s.all.end()) {
        set_error("serve: unknown request %lld", (long long)id);
        return MDZGPU_ERR_ARG;
    }
    const int state = it->second->state;
    if (state == MDZGPU_REQ_QUEUED || state == MDZGPU_REQ_RUNNING) {
        set_error("serve: request %lld has not finished", (long long)id);
        return MDZGPU_ERR_ARG;
    }
    srv->s.all.erase(it);
    return MDZGPU_OK;
}

int mdzgpu_serve_get_stats(mdzgpu_server* srv, mdzgpu_serve_stats* out)
{
    if (!srv || !out) {
        set_error("serve: null argument");
        return MDZGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(srv->s.mu);
    *out = srv->s.st;
    std::vector<double> v = srv->s.latencies;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) {
            // nearest-rank percentile
            size_t k = (size_t)ceil(q * (double)v.size());
            if (k < 1)
                k = 1;
            return v[std::min(k, v.size()) - 1];
        };
        out->latency_p50_ms = pct(0.50);
        out->latency_p99_ms = pct(0.99);
        out->latency_max_ms = v.back();
    }
    return MDZGPU_OK;
}

}  // extern "C"
