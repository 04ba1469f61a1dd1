// walk_whole.cu -- persistent step kernel for a graph resident in HBM.
//
// Replaces randomWalkKernel / randomWalkInsidePool[AllBatch]
// (src/WalkManager.h:229-274) for the case where every partition is cached on
// the device: walkers never need re-bucketing, so each one is stepped from
// creation to termination without leaving the SM.
//
// Design (GB300-first):
//  * Persistent grid: SMs x resident CTAs; each lane owns one walker at a time.
//  * Lazy walker creation: walker i is created from its index alone (start
//    vertex and, for PPR, its geometric length are pure functions of
//    (seed, run, i)), so no walker array is ever materialised.  A lane whose
//    walker ends takes the next index from a warp-aggregated atomic counter
//    (one atomic per warp refill), keeping every lane busy despite the
//    geometric length spread of PPR walks.
//  * Graph reads: rowptr[cur], rowptr[cur+1] (16 B) and col[e] (4 B) through
//    the read-only path; counters are u64 reductions resolved in L2.  Column
//    loads are evict-first, row offsets and counters evict-last (mem.cuh).
#include <algorithm>

#include "common.h"
#include "lt_core.cuh"
#include "mem.cuh"
#include "walk_whole.h"

namespace lt {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
// idle lanes a warp waits for before refilling them (all lanes: always): the
// refill sits on the warp's critical path and PPR's geometric walk lengths
// would otherwise trigger one nearly every iteration
constexpr int kRefillMin = 24;

struct Hints {
    uint64_t keep, stream;
};
__device__ __forceinline__ uint32_t ldg_u32(const uint32_t *p, const Hints &h) { return ld_nc_stream_u32(p, h.stream); }

// first edge and degree of v
template <int L>
__device__ __forceinline__ void row_range(const WholeArgs &a, uint32_t v, const Hints &h, uint64_t &first,
                                          uint64_t &deg)
{
    if (L == kLayoutPacked) {
        // the even words never change during a launch (only the counters
        // beside them do), so the read-only path serves them
        const uint32_t f = ld_nc_u32(a.rows + 2ull * v, h.keep);
        first = f;
        deg = ld_nc_u32(a.rows + 2ull * v + 2, h.keep) - f;
    } else if (L == kLayoutCompact) {
        const uint32_t f = ld_nc_u32(a.rowptr32 + v, h.keep);
        first = f;
        deg = ld_nc_u32(a.rowptr32 + v + 1, h.keep) - f;
    } else {
        first = ld_nc_u64(a.rowptr + v, h.keep);
        deg = ld_nc_u64(a.rowptr + v + 1, h.keep) - first;
    }
}

template <int L>
__device__ __forceinline__ void count1(const WholeArgs &a, uint32_t v, const Hints &h)
{
    if (L == kLayoutPacked)
        red_add1_u32(a.rows + 2ull * v + 1, h.keep);
    else if (L == kLayoutCompact)
        red_add1_u32(a.counts32 + v, h.keep);
    else
        red_add1_u64((unsigned long long *)(a.counts + v), h.keep);
}

template <int APP, int START, int C>
__global__ void __launch_bounds__(kWholeBlock) walk_whole_kernel(WholeArgs a)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const Hints h{l2_policy_evict_last(), l2_policy_evict_first()};

    uint32_t cur = 0, step = 0;
    uint64_t idx = 0;
    bool active = false;
    bool exhausted = false;
    uint32_t hop = 0;  // hops taken (walk app path position)
    uint64_t n_upd = 0, n_mov = 0, n_tel = 0;

    while (true) {
        const unsigned idle = __ballot_sync(kFull, !active);
        if (idle != 0u && !exhausted && (__popc(idle) >= kRefillMin || idle == kFull)) {
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd((unsigned long long *)a.next, (unsigned long long)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if (base + __popc(idle) >= a.W) exhausted = true;
            if (!active) {
                const uint64_t my = base + __popc(idle & lt_mask);
                if (my < a.W) {
                    idx = my;
                    cur = start_vertex(START, a.source, a.V, a.seed, a.run, idx);
                    if (APP == kPPR) {
                        step = ppr_length(a.seed, a.run, idx, a.thr);
                    } else {
                        step = a.length;
                    }
                    hop = 0;
                    if (APP == kWalk && a.paths) a.paths[idx * (uint64_t)(a.length + 1)] = cur;
                    active = true;
                }
            }
        }
        if (__ballot_sync(kFull, active) == 0u) {
            if (exhausted) break;
            continue;
        }
        if (!active) continue;

        const uint32_t s = step;
        n_upd++;
        if (APP == kPPR) {
            // app/ppr.cu:22-42
            if (s == 1) {
                count1<C>(a, cur, h);
                active = false;
            } else {
                step = s - 1;
                uint64_t first, deg;
                row_range<C>(a, cur, h, first, deg);
                if (deg > 0) {
                    const Rand4 r = walk_draw(a.seed, s, kTagStep, a.run, idx);
                    cur = ldg_u32(a.col + first + mod_u64(r64_of(r), deg), h);
                    n_mov++;
                } else {
                    count1<C>(a, cur, h);
                    active = false;
                }
            }
        } else if (APP == kPageRank) {
            // app/pagerank.cu:26-44; a vertex without out-edges teleports.
            count1<C>(a, cur, h);
            if (s == 1) {
                active = false;
            } else {
                step = s - 1;
                const Rand4 r = walk_draw(a.seed, s, kTagStep, a.run, idx);
                const uint64_t r64 = r64_of(r);
                bool tele = m53_of(r) >= a.thr;
                if (!tele) {
                    uint64_t first, deg;
                    row_range<C>(a, cur, h, first, deg);
                    if (deg > 0) {
                        cur = ldg_u32(a.col + first + mod_u64(r64, deg), h);
                        n_mov++;
                    } else {
                        tele = true;
                    }
                }
                if (tele) {
                    cur = (uint32_t)mod_u64(r64, a.V);
                    n_tel++;
                }
            }
        } else {
            // app/genericwalk.cu:22-32
            uint64_t first, deg;
            row_range<C>(a, cur, h, first, deg);
            uint32_t *path = a.paths ? a.paths + idx * (uint64_t)(a.length + 1) : nullptr;
            if (deg > 0) {
                const Rand4 r = walk_draw(a.seed, s, kTagStep, a.run, idx);
                cur = ldg_u32(a.col + first + mod_u64(r64_of(r), deg), h);
                n_mov++;
                hop++;
                if (path) path[hop] = cur;
                step = s - 1;
            } else {
                if (path) {
                    for (uint32_t h = hop + 1; h <= a.length; h++) path[h] = kInvalidNode;
                }
                step = 0;
            }
            if (step == 0) active = false;
        }
        if (!active && a.endpoints) a.endpoints[idx] = cur;
    }

    // Warp-reduce the statistics, one atomic per warp.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_upd += __shfl_down_sync(kFull, n_upd, o);
        n_mov += __shfl_down_sync(kFull, n_mov, o);
        n_tel += __shfl_down_sync(kFull, n_tel, o);
    }
    if (lane == 0 && a.stats) {
        atomicAdd((unsigned long long *)&a.stats[0], (unsigned long long)n_upd);
        atomicAdd((unsigned long long *)&a.stats[1], (unsigned long long)n_mov);
        atomicAdd((unsigned long long *)&a.stats[2], (unsigned long long)n_tel);
    }
}

template <int APP, int START, int C>
cudaError_t launch_t(const WholeArgs &a, int grid, cudaStream_t st)
{
    walk_whole_kernel<APP, START, C><<<grid, kWholeBlock, 0, st>>>(a);
    return cudaGetLastError();
}

template <int APP, int C>
cudaError_t launch_app(const WholeArgs &a, int start, int grid, cudaStream_t st)
{
    switch (start) {
    case kStartSource: return launch_t<APP, kStartSource, C>(a, grid, st);
    case kStartUniform: return launch_t<APP, kStartUniform, C>(a, grid, st);
    default: return launch_t<APP, kStartPerVertex, C>(a, grid, st);
    }
}

template <int APP, int START, int C>
int occupancy_t()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, walk_whole_kernel<APP, START, C>, kWholeBlock, 0);
    return n;
}

template <int C>
int occupancy_c(int app, int start)
{
    switch (app * 3 + start) {
    case 0: return occupancy_t<kPPR, kStartSource, C>();
    case 1: return occupancy_t<kPPR, kStartUniform, C>();
    case 2: return occupancy_t<kPPR, kStartPerVertex, C>();
    case 3: return occupancy_t<kPageRank, kStartSource, C>();
    case 4: return occupancy_t<kPageRank, kStartUniform, C>();
    case 5: return occupancy_t<kPageRank, kStartPerVertex, C>();
    case 6: return occupancy_t<kWalk, kStartSource, C>();
    case 7: return occupancy_t<kWalk, kStartUniform, C>();
    default: return occupancy_t<kWalk, kStartPerVertex, C>();
    }
}

}  // namespace

int whole_grid(int app, int start, int device, int ctas_per_sm, int layout)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int occ = layout == kLayoutPacked    ? occupancy_c<kLayoutPacked>(app, start)
              : layout == kLayoutCompact ? occupancy_c<kLayoutCompact>(app, start)
                                         : occupancy_c<kLayoutWide>(app, start);
    if (occ < 1) occ = 1;
    if (ctas_per_sm > 0 && ctas_per_sm < occ) occ = ctas_per_sm;
    return sms * occ;
}

template <int C>
cudaError_t launch_layout(const WholeArgs &a, int app, int start, int grid, cudaStream_t st)
{
    switch (app) {
    case kPPR: return launch_app<kPPR, C>(a, start, grid, st);
    case kPageRank: return launch_app<kPageRank, C>(a, start, grid, st);
    default: return launch_app<kWalk, C>(a, start, grid, st);
    }
}

cudaError_t launch_walk_whole(const WholeArgs &a, int app, int start, int grid, cudaStream_t st, int layout)
{
    if (layout == kLayoutPacked) return launch_layout<kLayoutPacked>(a, app, start, grid, st);
    if (layout == kLayoutCompact) return launch_layout<kLayoutCompact>(a, app, start, grid, st);
    return launch_layout<kLayoutWide>(a, app, start, grid, st);
}

namespace {

__global__ void mod_check_kernel(uint64_t n, const uint64_t *x, const uint64_t *d, uint64_t *out)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = d[i] ? mod_u64(x[i], d[i]) : ~0ull;
}

}  // namespace

}  // namespace lt

// The device build of the walk kernels' remainder, for checking it against
// native division (a zero divisor gives all ones).
extern "C" lt_status lt_mod_check_device(uint64_t n, const uint64_t *d_x, const uint64_t *d_d, uint64_t *d_out,
                                         void *stream)
{
    if (n == 0) return LT_OK;
    if (!d_x || !d_d || !d_out) return lt::fail(LT_ERR_INVALID, "null argument");
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, 152ull * 8);
    lt::mod_check_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(n, d_x, d_d, d_out);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of lt_walk_device.
//
// Some callers cannot allocate device memory: plugins handed fixed input and
// output buffers by a host framework that owns every allocation, and
// processes whose device memory another allocator has reserved in full.
// lt_walk_device asks them for a scratch buffer; this entry point needs none.  Its scratch (the
// next-walker counter of the step kernel) lives in the file-scope array below,
// which every GPU that loads this library holds until the process exits.
//
// The array is kNoAllocScratchBytes (256 B); the step kernel's scratch does not
// grow with the graph or the walker count (one 8-byte counter inside a
// walk_scratch_bytes()-byte block), and a call whose scratch need exceeds the
// array is rejected with LT_ERR_CAPACITY.
//
// All calls share the one array: it keeps the previous call's contents, so the
// counter is cleared on the caller's stream before each launch, and two calls
// whose kernels overlap on the GPU (different streams, no ordering between
// them) race on the counter and produce wrong results.  Order such calls on one
// stream.
//
// The device address of the array is looked up once per device, on the first
// call made with that device current (cudaGetSymbolAddress), and kept for the
// life of the process; make that first call before any stream capture begins.
// The kept address assumes the device's primary context is never reset: after
// a cudaDeviceReset the module is loaded again and the address may be stale.
// ---------------------------------------------------------------------------

#include <mutex>

#include "common.h"
#include "engine.h"

namespace lt {
namespace {

constexpr size_t kNoAllocScratchBytes = 256;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kNoAllocMaxDevices] = {};

lt_status noalloc_scratch(void **out)
{
    int device = 0;
    LT_CUDA_TRY(cudaGetDevice(&device));
    if (device < 0 || device >= kNoAllocMaxDevices)
        return fail(LT_ERR_UNSUPPORTED, "device ordinal %d is beyond the %d devices the static scratch tracks", device,
                    kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (err != cudaSuccess || !p)
            return fail(LT_ERR_CUDA, "cudaGetSymbolAddress of the static walk scratch failed on device %d: %s",
                        device, cudaGetErrorString(err));
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
    return LT_OK;
}

}  // namespace
}  // namespace lt

extern "C" lt_status lt_walk_device_noalloc(int app, int start_mode, const uint64_t *d_rowptr, const uint32_t *d_col,
                                            uint32_t num_nodes, uint32_t source, uint64_t num_walkers,
                                            uint32_t length, float prob, uint32_t run, uint64_t seed,
                                            uint64_t *d_counts, uint32_t *d_endpoints, uint32_t *d_paths,
                                            uint64_t *d_stats, void *stream)
{
    const size_t need = lt::walk_scratch_bytes();
    if (need > lt::kNoAllocScratchBytes)
        return lt::fail(LT_ERR_CAPACITY, "the step kernel needs %zu scratch bytes; the static array holds %zu", need,
                        lt::kNoAllocScratchBytes);
    void *scratch = nullptr;
    LT_TRY(lt::noalloc_scratch(&scratch));
    return lt::walk_device(app, start_mode, d_rowptr, d_col, num_nodes, source, num_walkers, length, prob, run, seed,
                           d_counts, d_endpoints, d_paths, scratch, d_stats, (cudaStream_t)stream, 0);
}
