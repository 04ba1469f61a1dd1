// rmat.cu -- seeded RMAT graph generator on the GPU.
//
// The reference reads its datasets from disk (tools/convert_from_txt.cc); the
// synthetic RMAT graphs stand in for them.  The generator is written so that
// the CSR comes out directly, without sorting an edge list:
//   1. the source of edge i is drawn bit by bit (level l uses 16-bit lane l
//      of Philox(ctr = (i lo, i hi, 0x10, l / 8)); bit = lane >= T_src) and
//      counted into out-degrees;  the multiset of sources is exactly that of
//      RMAT;
//   2. rowptr = exclusive scan of the out-degrees;
//   3. the k-th out-edge of u gets its destination from the RMAT conditional
//      given u's bits (lane l of Philox(ctr = (u, k, 0x11, l / 8)); bit =
//      lane >= (bit_l(u) ? T_d1 : T_d0)), so col is a pure function of (u, k);
//   4. vertices with no in- and no out-edges are removed keeping order
//      (tools/rm_isolated_vertices.cc:70-87).
// Every step is integer-only, so the CPU restatement produces the same bytes.
#include <cstdio>

#include "common.h"
#include "graph.h"
#include "lt_core.cuh"
#include "scan.cuh"

namespace lt {

namespace {

constexpr int kGenBlock = 256;

__device__ __forceinline__ uint32_t rmat_src(uint64_t seed, uint64_t i, int scale, uint32_t t_src)
{
    uint32_t v = 0;
    Rand4 r{};
    for (int l = 0; l < scale; l++) {
        if ((l & 7) == 0)
            r = philox4x32_10((uint32_t)i, (uint32_t)(i >> 32), kTagRmatSrc, (uint32_t)(l >> 3), (uint32_t)seed,
                              (uint32_t)(seed >> 32));
        v = (v << 1) | (lane16(r, l & 7) >= t_src ? 1u : 0u);
    }
    return v;
}

__device__ __forceinline__ uint32_t rmat_dst(uint64_t seed, uint32_t u, uint32_t k, int scale, uint32_t t_d0,
                                             uint32_t t_d1)
{
    uint32_t v = 0;
    Rand4 r{};
    for (int l = 0; l < scale; l++) {
        if ((l & 7) == 0)
            r = philox4x32_10(u, k, kTagRmatDst, (uint32_t)(l >> 3), (uint32_t)seed, (uint32_t)(seed >> 32));
        const uint32_t sbit = (u >> (scale - 1 - l)) & 1u;
        v = (v << 1) | (lane16(r, l & 7) >= (sbit ? t_d1 : t_d0) ? 1u : 0u);
    }
    return v;
}

__global__ void __launch_bounds__(kGenBlock) degrees_kernel(uint64_t E, uint64_t seed, int scale, uint32_t t_src,
                                                            uint32_t *deg)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < E; i += stride)
        atomicAdd(&deg[rmat_src(seed, i, scale, t_src)], 1u);
}

// One warp per 32 consecutive vertices; lanes stride over the warp's edge range
// and find their vertex by a binary search over the 33 row offsets held in
// lane registers.
__global__ void __launch_bounds__(kGenBlock) fill_kernel(uint64_t V0, const uint64_t *rowptr, uint64_t seed, int scale,
                                                         uint32_t t_d0, uint32_t t_d1, uint32_t *col)
{
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; w * 32 < V0; w += warps) {
        const uint64_t u0 = w * 32;
        const uint64_t my_u = u0 + lane;
        const uint64_t my_off = rowptr[my_u < V0 ? my_u : V0];
        const uint64_t end = rowptr[u0 + 32 < V0 ? u0 + 32 : V0];
        const uint64_t begin = __shfl_sync(0xFFFFFFFFu, my_off, 0);
        for (uint64_t e = begin + lane; __any_sync(0xFFFFFFFFu, e < end); e += 32) {
            // largest j with off[j] <= e (off[j] = row start of vertex u0 + j)
            int lo = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const uint64_t probe = __shfl_sync(0xFFFFFFFFu, my_off, lo + step);
                if (lo + step < 32 && u0 + lo + step <= V0 && probe <= e) lo += step;
            }
            // skip vertices with no edges that share the same start offset
            if (e < end) {
                const uint64_t u = u0 + lo;
                const uint64_t k = e - rowptr[u];
                col[e] = rmat_dst(seed, (uint32_t)u, (uint32_t)k, scale, t_d0, t_d1);
            }
        }
    }
}

__global__ void mark_present(uint64_t V0, const uint32_t *deg, uint32_t *present)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V0; v += stride) present[v] = deg[v] > 0;
}

__global__ void mark_targets(uint64_t E, const uint32_t *col, uint32_t *present)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) present[col[e]] = 1u;
}

__global__ void compact_rowptr(uint64_t V0, const uint32_t *present, const uint32_t *newid, const uint64_t *rowptr,
                               uint64_t *rowptr2)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= V0; v += stride) {
        if (v == V0)
            rowptr2[newid[V0]] = rowptr[V0];
        else if (present[v])
            rowptr2[newid[v]] = rowptr[v];
    }
}

__global__ void remap_col(uint64_t E, const uint32_t *newid, uint32_t *col)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) col[e] = newid[col[e]];
}

struct DevBufs {
    void *p[6] = {};
    ~DevBufs()
    {
        for (void *q : p)
            if (q) cudaFree(q);
    }
};

}  // namespace

uint32_t rmat_q16(double p) { return (uint32_t)(p * 65536.0 + 0.5); }

lt_status generate_rmat(int device, uint32_t scale, uint64_t E, double a, double b, double c, double d, uint64_t seed,
                        lt_graph &g)
{
    if (scale < 1 || scale > 31) return fail(LT_ERR_INVALID, "RMAT scale %u outside [1, 31]", scale);
    if (!(a >= 0 && b >= 0 && c >= 0 && d >= 0) || a + b <= 0 || c + d <= 0)
        return fail(LT_ERR_INVALID, "RMAT probabilities must be non-negative with a+b > 0 and c+d > 0");
    const uint32_t t_src = rmat_q16(a + b), t_d0 = rmat_q16(a / (a + b)), t_d1 = rmat_q16(c / (c + d));
    LT_CUDA_TRY(cudaSetDevice(device));
    const uint64_t V0 = 1ull << scale;
    int sms = 0;
    LT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int grid = sms * 8;
    cudaStream_t st = 0;

    DevBufs B;
    uint32_t *d_deg, *d_col, *d_present, *d_newid;
    uint64_t *d_rowptr, *d_tmp;
    LT_CUDA_TRY(cudaMalloc(&B.p[0], 4 * V0));
    d_deg = (uint32_t *)B.p[0];
    LT_CUDA_TRY(cudaMalloc(&B.p[1], 8 * (V0 + 1)));
    d_rowptr = (uint64_t *)B.p[1];
    LT_CUDA_TRY(cudaMalloc(&B.p[2], 4 * (E ? E : 1)));
    d_col = (uint32_t *)B.p[2];
    LT_CUDA_TRY(cudaMalloc(&B.p[3], 8 * scan_tmp_elems(V0 + 1)));
    d_tmp = (uint64_t *)B.p[3];

    LT_CUDA_TRY(cudaMemsetAsync(d_deg, 0, 4 * V0, st));
    degrees_kernel<<<grid, kGenBlock, 0, st>>>(E, seed, (int)scale, t_src, d_deg);
    LT_CUDA_TRY(cudaGetLastError());
    LT_CUDA_TRY((exclusive_scan<uint32_t, uint64_t>(d_deg, V0, d_rowptr, d_tmp, st)));
    fill_kernel<<<grid, kGenBlock, 0, st>>>(V0, d_rowptr, seed, (int)scale, t_d0, t_d1, d_col);
    LT_CUDA_TRY(cudaGetLastError());

    // isolated-vertex removal: present = out-degree > 0 or some in-edge.
    d_present = d_deg;  // reuse: deg is not needed after the flags are set
    mark_present<<<grid, kGenBlock, 0, st>>>(V0, d_deg, d_present);
    mark_targets<<<grid, kGenBlock, 0, st>>>(E, d_col, d_present);
    LT_CUDA_TRY(cudaGetLastError());
    LT_CUDA_TRY(cudaMalloc(&B.p[4], 4 * (V0 + 1)));
    d_newid = (uint32_t *)B.p[4];
    uint32_t *d_tmp32 = (uint32_t *)d_tmp;
    LT_CUDA_TRY((exclusive_scan<uint32_t, uint32_t>(d_present, V0, d_newid, d_tmp32, st)));
    uint32_t V = 0;
    LT_CUDA_TRY(cudaMemcpyAsync(&V, d_newid + V0, 4, cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaStreamSynchronize(st));
    LT_CUDA_TRY(cudaMalloc(&B.p[5], 8 * ((uint64_t)V + 1)));
    uint64_t *d_rowptr2 = (uint64_t *)B.p[5];
    compact_rowptr<<<grid, kGenBlock, 0, st>>>(V0, d_present, d_newid, d_rowptr, d_rowptr2);
    remap_col<<<grid, kGenBlock, 0, st>>>(E, d_newid, d_col);
    LT_CUDA_TRY(cudaGetLastError());

    g.V = V;
    g.E = E;
    LT_TRY(host_alloc(g.rowptr_buf, 8ull * ((uint64_t)V + 1), true));
    LT_TRY(host_alloc(g.col_buf, 4ull * E, true));
    LT_CUDA_TRY(cudaMemcpyAsync(g.rowptr_mut(), d_rowptr2, 8ull * ((uint64_t)V + 1), cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaMemcpyAsync(g.col_mut(), d_col, 4ull * E, cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaStreamSynchronize(st));
    return LT_OK;
}

}  // namespace lt
