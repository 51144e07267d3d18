// Allocation-free chi-squared reduction: galario_reduce_chi2_noalloc_d.
//
// Why it exists: some callers cannot let this library allocate GPU memory.
// A sampler embedded in a larger GPU application often runs with all device
// memory owned by another allocator (PyTorch's caching allocator, a memory
// pool sized at start-up), so a cudaMalloc from here can fail or fragment that
// pool; and cudaFree synchronises the whole device, which a caller driving
// many asynchronous streams cannot afford inside its loop.  This entry point
// therefore takes only caller-owned device buffers and uses, as its scratch,
// a fixed array that is part of this library's device image.
//
// Scratch: g_noalloc_scratch below, 4096 per-block partial sums (32 KiB) and a
// block-completion counter.  Every GPU on which the library is loaded keeps
// this array until the process exits.  Every call uses the same array, and
// the array keeps what the last call left in it: each call clears the counter
// before its kernel runs, and the partial sums are overwritten before they are
// read.  Because the array is shared, two calls whose kernels overlap on the
// GPU (different streams, no ordering between them) race and give wrong
// results; order such calls on one stream or synchronise between them.
//
// Limit: one thread block reduces 4096 visibilities and there are 4096
// partial sums, so nd may be at most 4096 * 4096 = 16,777,216; larger nd is
// rejected with GALARIO_EINVAL.
//
// Set-up: the first call on each device, with that device current, looks up
// the device address of the array (cudaGetSymbolAddress) and caches it; make
// that first call before any stream capture on the device.  galario_cleanup()
// forgets the cached addresses (call it after a cudaDeviceReset, which reloads
// the library's device image, possibly elsewhere).
//
// vis_dev holds nd interleaved (re, im) doubles and is read 16 bytes at a
// time, so it must be 16-byte aligned (a complex128 array is; a view that
// starts at an odd double is not): a misaligned pointer is rejected with
// GALARIO_EINVAL before anything is enqueued.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/galario_gb300.h"

namespace gbg {
void set_error_message(const std::string& msg);  // gb_api.cu: backs galario_last_error()
}

namespace {

constexpr int kThreads = 256;
constexpr int kItemsPerThread = 16;
constexpr int kItemsPerBlock = kThreads * kItemsPerThread;  // 4096
constexpr int kMaxBlocks = 4096;
constexpr long long kMaxNd = (long long)kItemsPerBlock * kMaxBlocks;  // 16,777,216
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    double partials[kMaxBlocks];
    unsigned int ticket;  // blocks that have finished; must be 0 when a call starts
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_setup_mu;
NoAllocScratch* g_scratch_ptr[kMaxDevices] = {};

__device__ __forceinline__ double block_sum_256(double x, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < kThreads / 32; ++q) s += sh[q];
    return s;  // valid in thread 0
}

// chi2 = sum w * |vis - (re + i im)|^2 in FP64 (the reduction of the
// reference's reduce_chi2, src/galario.cpp:1504-1538).  Block b reduces
// items [4096 b, 4096 (b+1)); the last block to finish adds the partial sums
// in a fixed order, so the result does not depend on scheduling.
__global__ void __launch_bounds__(kThreads) reduce_chi2_noalloc_kernel(const double* __restrict__ re,
                                                                       const double* __restrict__ im,
                                                                       const double2* __restrict__ vis,
                                                                       const double* __restrict__ w, int nd,
                                                                       NoAllocScratch* scratch,
                                                                       double* __restrict__ chi2_out) {
    __shared__ double sh[kThreads / 32];
    __shared__ double sh2[kThreads / 32];
    __shared__ bool last;
    const long long base = (long long)blockIdx.x * kItemsPerBlock;
    double acc = 0.0;
#pragma unroll 4
    for (int j = 0; j < kItemsPerThread; ++j) {
        const long long i = base + (long long)j * kThreads + threadIdx.x;
        if (i < nd) {
            const double2 z = __ldg(&vis[i]);
            const double dr = z.x - __ldg(&re[i]), di = z.y - __ldg(&im[i]);
            acc += __ldg(&w[i]) * (dr * dr + di * di);
        }
    }
    const double tot = block_sum_256(acc, sh);
    if (threadIdx.x == 0) {
        scratch->partials[blockIdx.x] = tot;
        __threadfence();
        last = (atomicAdd(&scratch->ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const volatile double* p = scratch->partials;
    double s = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += kThreads) s += p[b];
    s = block_sum_256(s, sh2);
    if (threadIdx.x == 0) {
        *chi2_out = s;
        scratch->ticket = 0u;
    }
}

// Device address of the scratch array for the current device (looked up once per device).
cudaError_t scratch_for_current_device(NoAllocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<NoAllocScratch*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

int fail(int status, const std::string& msg) {
    gbg::set_error_message(msg);
    return status;
}

}  // namespace

namespace gbg {
// galario_cleanup (gb_api.cu): forget the per-device scratch addresses
void noalloc_forget_scratch() {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    for (auto& p : g_scratch_ptr) p = nullptr;
}
}  // namespace gbg

extern "C" __attribute__((visibility("default"))) int galario_reduce_chi2_noalloc_d(
    int nd, const double* re_dev, const double* im_dev, const double* vis_dev, const double* w_dev, double* chi2_dev,
    void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nd < 0) return fail(GALARIO_EINVAL, "Error in reduce_chi2_noalloc: nd = " + std::to_string(nd) + " is negative");
    if ((long long)nd > kMaxNd)
        return fail(GALARIO_EINVAL, "Error in reduce_chi2_noalloc: nd = " + std::to_string(nd) +
                                        " exceeds the maximum of " + std::to_string(kMaxNd) +
                                        " visibilities of the allocation-free entry point");
    if (!chi2_dev) return fail(GALARIO_EINVAL, "Error in reduce_chi2_noalloc: chi2_dev is NULL");
    if (nd == 0) {
        const cudaError_t e = cudaMemsetAsync(chi2_dev, 0, sizeof(double), s);
        if (e != cudaSuccess) return fail(GALARIO_ERUNTIME, std::string("Error in cuda: ") + cudaGetErrorString(e));
        return GALARIO_OK;
    }
    if (!re_dev || !im_dev || !vis_dev || !w_dev)
        return fail(GALARIO_EINVAL, "Error in reduce_chi2_noalloc: a device pointer is NULL");
    if ((reinterpret_cast<std::uintptr_t>(vis_dev) & 15u) != 0)
        return fail(GALARIO_EINVAL, "Error in reduce_chi2_noalloc: vis_dev must be 16-byte aligned "
                                    "(nd interleaved (re, im) doubles)");
    NoAllocScratch* scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess)
        return fail(GALARIO_ERUNTIME, std::string("Error in cuda (cudaGetSymbolAddress): ") + cudaGetErrorString(e));
    // the completion counter must start at zero whatever an earlier call left behind
    e = cudaMemsetAsync(&scratch->ticket, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return fail(GALARIO_ERUNTIME, std::string("Error in cuda: ") + cudaGetErrorString(e));
    const int blocks = (int)(((long long)nd + kItemsPerBlock - 1) / kItemsPerBlock);
    reduce_chi2_noalloc_kernel<<<blocks, kThreads, 0, s>>>(re_dev, im_dev, reinterpret_cast<const double2*>(vis_dev),
                                                            w_dev, nd, scratch, chi2_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(GALARIO_ERUNTIME, std::string("Error in cuda: ") + cudaGetErrorString(e));
    return GALARIO_OK;
}
