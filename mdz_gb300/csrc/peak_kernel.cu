// Pipe-throughput microbenchmarks: the roofline denominators for the
// escape-time kernels, which are bound by the FP32, INT32 (IMAD) or FP64
// pipes rather than by HBM or the tensor cores.  Each thread runs 8
// independent dependency chains so the pipe, not latency, is the limit.
#include "internal.h"

namespace mdz {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) ffma_peak(float* sink, float a, float b)
{
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        x[c] = threadIdx.x * 1e-7f + c;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += x[c];
    if (s == 1234.5f)
        sink[0] = s;
}

__global__ void __launch_bounds__(256) imad_peak(unsigned* sink, unsigned a, unsigned b)
{
    unsigned x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        x[c] = threadIdx.x + c;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[c]) : "r"(a), "r"(b));
    }
    unsigned s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s ^= x[c];
    if (s == 0x12345u)
        sink[0] = s;
}

__global__ void __launch_bounds__(256) dmul_peak(double* sink, double a, double b)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        x[c] = threadIdx.x * 1e-9 + c;
    for (int i = 0; i < kIters / 8; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            x[c] = __dadd_rn(__dmul_rn(x[c], a), b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += x[c];
    if (s == 1234.5)
        sink[0] = s;
}

}  // namespace
}  // namespace mdz

using namespace mdz;

extern "C" int mdzgpu_measure_peak(int device, int kind, double* ops_per_s)
{
    if (!ops_per_s)
        return MDZGPU_ERR_ARG;
    MDZ_CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop;
    MDZ_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    void* sink = nullptr;
    MDZ_CUDA_TRY(cudaMalloc(&sink, 64));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = prop.multiProcessorCount * 8;
    const int threads = 256;
    double ops = 0.0;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (kind == 0) {
            ffma_peak<<<blocks, threads>>>((float*)sink, 0.999f, 1e-3f);
            ops = (double)blocks * threads * kIters * kChains;
        } else if (kind == 1) {
            imad_peak<<<blocks, threads>>>((unsigned*)sink, 1664525u, 1013904223u);
            ops = (double)blocks * threads * kIters * kChains;
        } else {
            dmul_peak<<<blocks, threads>>>((double*)sink, 0.999, 1e-3);
            ops = (double)blocks * threads * (kIters / 8) * kChains * 2;
        }
        cudaEventRecord(e1);
        cudaError_t err = cudaEventSynchronize(e1);
        if (err != cudaSuccess) {
            cudaFree(sink);
            set_error("peak kernel: %s", cudaGetErrorString(err));
            return MDZGPU_ERR_CUDA;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best)
            best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    *ops_per_s = ops / (best * 1e-3);
    return MDZGPU_OK;
}
