// scan.cuh -- device-wide exclusive prefix sum (three passes: tile sums, a
// single-CTA scan of the tile sums, tile scans with carry-in).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lt {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

namespace scan_detail {

// Exclusive prefix sum of one value per thread over a block of BLOCK threads
// (a multiple of 32, at most 1024); *total receives the block's sum.
template <typename T, int BLOCK = kScanBlock>
__device__ __forceinline__ T block_exclusive(T v, T *warp_tot, T *total)
{
    static_assert(BLOCK % 32 == 0 && BLOCK <= 1024, "block of whole warps, at most 1024 threads");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T n = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += n;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T w = lane < BLOCK / 32 ? warp_tot[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T n = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= o) wi += n;
        }
        if (lane < BLOCK / 32) warp_tot[lane] = wi - w;
        if (lane == BLOCK / 32 - 1) *total = wi;
    }
    __syncthreads();
    const T r = incl - v + warp_tot[wid];
    __syncthreads();
    return r;
}

template <typename In, typename Out>
__global__ void __launch_bounds__(kScanBlock) tile_sums(const In *in, uint64_t n, Out *sums)
{
    __shared__ Out warp_tot[kScanBlock / 32];
    __shared__ Out total;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    Out s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) s += (Out)in[base + k];
    block_exclusive<Out>(s, warp_tot, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <typename Out>
__global__ void __launch_bounds__(kScanBlock) scan_sums(Out *sums, uint64_t nb, Out *grand_total)
{
    __shared__ Out warp_tot[kScanBlock / 32];
    __shared__ Out total;
    Out carry = 0;
    for (uint64_t base = 0; base < nb; base += kScanBlock) {
        const uint64_t i = base + threadIdx.x;
        const Out v = i < nb ? sums[i] : Out(0);
        const Out ex = block_exclusive<Out>(v, warp_tot, &total);
        if (i < nb) sums[i] = ex + carry;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

template <typename In, typename Out>
__global__ void __launch_bounds__(kScanBlock) tile_scan(const In *in, uint64_t n, const Out *sums, Out *out)
{
    __shared__ Out warp_tot[kScanBlock / 32];
    __shared__ Out total;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    Out v[kScanItems];
    Out s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? (Out)in[base + k] : Out(0);
        s += v[k];
    }
    Out run = block_exclusive<Out>(s, warp_tot, &total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

}  // namespace scan_detail

// out[i] = sum(in[0..i)) for i in [0, n]; out has n+1 entries (out[n] = total).
// tmp must hold ceil(n / kScanTile) + 1 Out values.  In and out may not alias.
template <typename In, typename Out>
cudaError_t exclusive_scan(const In *in, uint64_t n, Out *out, Out *tmp, cudaStream_t st)
{
    const uint64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) return cudaMemsetAsync(out, 0, sizeof(Out), st);
    scan_detail::tile_sums<In, Out><<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, tmp);
    scan_detail::scan_sums<Out><<<1, kScanBlock, 0, st>>>(tmp, nb, out + n);
    scan_detail::tile_scan<In, Out><<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, tmp, out);
    return cudaGetLastError();
}

inline size_t scan_tmp_elems(uint64_t n) { return (size_t)((n + kScanTile - 1) / kScanTile) + 1; }

}  // namespace lt
