// Measurement helper (no counterpart in the reference): the FP64 fused
// multiply-add rate of the current GPU, the denominator of the FP64-pipe
// roofline of the double-precision kernels (on GB300 FP64 arithmetic, not HBM,
// bounds them).
//
// Every thread runs kChains independent FMA chains (x = x * a + b) for
// `iters` iterations, so the pipe never waits on a dependency; the grid is
// 8 blocks of 256 threads per SM.  The chains' results are summed into one
// double per block so that the compiler keeps the work.  Two flops per FMA.
#include <cuda_runtime.h>

#include <string>

#include "../../include/galario_gb300.h"

namespace gbg {
void set_error_message(const std::string& msg);  // gb_api.cu
}

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) fp64_fma_kernel(int iters, double a, double b, double* __restrict__ out) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c) * 1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&out[blockIdx.x], s);
}

int fail(const std::string& msg) {
    gbg::set_error_message(msg);
    return GALARIO_ERUNTIME;
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int galario_measure_fp64_peak(double* gflops) {
    if (!gflops) {
        gbg::set_error_message("Error in measure_fp64_peak: gflops is NULL");
        return GALARIO_EINVAL;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(std::string("Error in cuda: ") + cudaGetErrorString(e));
    const int blocks = 8 * sms;
    const int iters = 4096;
    double* out = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaStream_t s = nullptr;
    float best = 1e30f;
    e = cudaMalloc(&out, sizeof(double) * blocks);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e == cudaSuccess) e = cudaMemsetAsync(out, 0, sizeof(double) * blocks, s);
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {  // the first launch warms up; best of the rest
        cudaEventRecord(t0, s);
        fp64_fma_kernel<<<blocks, kThreads, 0, s>>>(iters, 0.999999, 1e-7, out);
        cudaEventRecord(t1, s);
        e = cudaEventSynchronize(t1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
        if (e == cudaSuccess && rep > 0 && ms < best) best = ms;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    if (e != cudaSuccess) return fail(std::string("Error in cuda: ") + cudaGetErrorString(e));
    const double flops = 2.0 * kChains * (double)iters * (double)blocks * kThreads;
    *gflops = flops / (best * 1e-3) / 1e9;
    return GALARIO_OK;
}
