// lg_peak.cu -- FP64/FP32 pipe throughput microbenchmark (measurement only).
//
// The FP64 leap-frog path is bound by the FP64 pipe, not by HBM, so its
// roofline needs the measured FP64 instruction rate of the part, which the
// copy/GEMM peaks do not give.  Each thread runs kChains independent
// dependency chains of one operation; enough warps are launched to fill every
// SM, so the rate measured is the pipe's issue throughput.
#include <cuda_runtime.h>

#include "lulesh_gb300.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <int OP, typename T>
__global__ void __launch_bounds__(256) k_pipe(T *out, T seed)
{
    T a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = seed + T(threadIdx.x * kChains + c) * T(1e-9);
    const T m = seed * T(0.999999), b = T(1e-12);
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) {
            if (OP == 0)
                a[c] = a[c] * m + b;  // one FMA
            else if (OP == 1)
                a[c] = a[c] + b;
            else
                a[c] = a[c] * m;
        }
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += a[c];
    if (s == T(-1)) out[blockIdx.x] = s;  // keeps the chains live
}

template <int OP, typename T>
int measure(double *ginst)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LG_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return LG_ERR_CUDA;
    const int blocks = sms * 8, threads = 256;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks) != cudaSuccess) return LG_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_pipe<OP, T><<<blocks, threads>>>(out, T(1.0));  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        k_pipe<OP, T><<<blocks, threads>>>(out, T(1.0));
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return LG_ERR_CUDA;
    const double inst = (double)blocks * threads * kChains * (double)kIters;
    *ginst = inst / (best * 1e-3) / 1e9;
    return LG_OK;
}

}  // namespace

extern "C" int lg_measure_pipe(int op, int fp32, double *ginst_per_s)
{
    if (!ginst_per_s || op < 0 || op > 2) return LG_ERR_INVALID;
    if (fp32) {
        switch (op) {
        case 0: return measure<0, float>(ginst_per_s);
        case 1: return measure<1, float>(ginst_per_s);
        default: return measure<2, float>(ginst_per_s);
        }
    }
    switch (op) {
    case 0: return measure<0, double>(ginst_per_s);
    case 1: return measure<1, double>(ginst_per_s);
    default: return measure<2, double>(ginst_per_s);
    }
}
