// probe.cu -- the host-link ceiling of zero-copy hops.
//
// A zero-copy hop reads one 4-byte column entry from pinned host memory; the
// link moves the whole 32-byte sector holding it (measured with ncu: 31.9 B
// per hop).  lt_host_gather_gbs measures how many such sectors the GPU can
// pull per second when every SM issues independent random reads: the roofline
// of the zero-copy step kernels (the copy engine's rate, lt_host_link_gbs, is
// the roofline of partition loads).
#include <algorithm>

#include "common.h"
#include "mem.cuh"

namespace lt {
namespace {

constexpr int kGatherIlp = 8;  // independent reads in flight per thread

__global__ void __launch_bounds__(256) host_gather_kernel(const uint32_t *host, uint64_t n_words, uint32_t iters,
                                                          unsigned long long *sink)
{
    uint64_t x = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
    const uint64_t stream = l2_policy_evict_first();  // the column loads of the step kernels
    uint32_t acc = 0;
    for (uint32_t i = 0; i < iters; i++) {
        uint32_t v[kGatherIlp];
#pragma unroll
        for (int k = 0; k < kGatherIlp; k++) {
            x = x * 6364136223846793005ull + 1442695040888963407ull;  // 64-bit LCG (Knuth's MMIX constants)
            v[k] = ld_nc_stream_u32(host + (x >> 24) % n_words, stream);
        }
#pragma unroll
        for (int k = 0; k < kGatherIlp; k++) acc += v[k];
    }
    if (acc == 0x9E3779B9u) atomicAdd(sink, 1ull);  // keeps the reads live
}

}  // namespace
}  // namespace lt

// Random 32-byte-sector read rate from mapped pinned host memory, in GB/s of
// sectors (best of 5 launches over a buffer of `bytes`, 0 = 2 GiB, far beyond
// L2; the column loads of the step kernels, evict-first and not allocated in
// L1).  The rate depends on how much host memory the reads spread over (on
// this machine about 130 GB/s up to 16 GiB, 1-2 GB/s at 32 GiB), which is
// why zero-copy reads go in bounded groups.
extern "C" lt_status lt_host_gather_gbs(int device, uint64_t bytes, double *gbs)
{
    using namespace lt;
    if (!gbs) return fail(LT_ERR_INVALID, "null argument");
    LT_CUDA_TRY(cudaSetDevice(device));
    if (bytes == 0) bytes = 2ull << 30;
    if (bytes < (64ull << 20)) return fail(LT_ERR_INVALID, "gather probe buffer below 64 MiB");
    const uint64_t n_words = bytes / 4;
    void *h = nullptr, *hd = nullptr;
    unsigned long long *sink = nullptr;
    LT_CUDA_TRY(cudaHostAlloc(&h, bytes, cudaHostAllocMapped | cudaHostAllocPortable));
    lt_status st = LT_OK;
    if (cudaHostGetDevicePointer(&hd, h, 0) != cudaSuccess || cudaMalloc(&sink, 8) != cudaSuccess) {
        cudaGetLastError();
        st = fail(LT_ERR_CUDA, "mapped pinned buffer for the gather probe");
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const unsigned blocks = (unsigned)std::max(1, sms * 8);
    // 152 x 8 x 256 threads x 16 x 8 reads = 40 M sectors (1.3 GB) per launch:
    // 10 ms at 130 GB/s, under a second at the slowest rate measured
    const uint32_t iters = 16;
    double best = 0;
    cudaEvent_t a = nullptr, b = nullptr;
    if (st == LT_OK) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        for (int r = 0; r < 6; r++) {
            cudaEventRecord(a, 0);
            host_gather_kernel<<<blocks, 256>>>((const uint32_t *)hd, n_words, iters, sink);
            cudaEventRecord(b, 0);
            if (cudaEventSynchronize(b) != cudaSuccess) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            const double sectors = (double)blocks * 256 * iters * kGatherIlp;
            if (r > 0 && ms > 0) best = std::max(best, sectors * 32.0 / (ms / 1e3) / 1e9);
        }
        if (cudaGetLastError() != cudaSuccess) st = fail(LT_ERR_CUDA, "gather probe failed");
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    if (sink) cudaFree(sink);
    cudaFreeHost(h);
    *gbs = best;
    return st;
}
