// batch.cu -- batched multi-source PPR: one persistent walk launch for many
// queries, per-query hash aggregation of endpoint counts, compaction, all
// captured in one CUDA graph and replayed per batch.
//
// Pipeline (sizes are read from a device header, so launch shapes are fixed
// and the captured graph is reused for every batch that fits the buffers):
//   prep    : one CTA; woff = scan(walkers), table capacity per query
//             cap = next_pow2(max(walkers << load_shift, 32)), toff = scan(cap);
//   clear   : tables to empty;
//   walk    : persistent, warp-aggregated refill over the global walker
//             ordinal; a walker finds its query by binary search over woff
//             (shared memory), is created from (query seed, index) and stepped
//             with the PPR semantics of app/ppr.cu:22-42 to its endpoint, which
//             is added to the query's table (linear probing, u32 counts);
//   count   : one CTA per query counts its occupied slots;
//   offsets : exclusive scan of the counts;
//   compact : one CTA per query writes (vertex, count) pairs in slot order.
#include "batch.h"

#include <algorithm>
#include <chrono>
#include <vector>

#include "engine.h"
#include "lt_core.cuh"
#include "mem.cuh"
#include "scan.cuh"

namespace lt {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kEmpty = 0xFFFFFFFFu;
// A warp refills its idle lanes only once at least this many are idle (or
// all of them): a refill (query lookup, walk-length draws) runs on the
// warp's critical path, and PPR's geometric lengths would otherwise make
// nearly every iteration a refill.  24 of 32 measured best on c3
// (70.5 -> 25.0 ms per batch; 16: 31.3, 32: 29.5).
constexpr int kRefillMin = 24;
constexpr uint32_t kSmemQueries = 8192;  // up to this many u32 walker offsets go to shared memory
constexpr int kPrepThreads = 1024;
constexpr int kRowThreads = 256;

struct Header {
    unsigned long long n;        // queries
    unsigned long long W;        // walkers in the batch
    unsigned long long T;        // table slots
    unsigned long long next;     // walk kernel: next ordinal
    unsigned long long error;    // a probe sequence ran past the table (never by construction)
    unsigned long long stats[3]; // updates, moves, -
};

struct BatchArgs {
    const uint32_t *n_dev;   // queries in the batch (written by the host before each launch)
    uint32_t smem_queries;   // walker offsets kept in shared memory when n <= smem_queries
    const uint64_t *rowptr;
    const uint32_t *rowptr32;  // compact row offsets when E < 2^32 (else null)
    const uint32_t *col;
    uint32_t V;
    uint64_t thr;
    Header *hdr;
    const uint32_t *src;
    const uint64_t *walkers;
    const uint64_t *seeds;
    uint64_t *woff;      // n+1
    uint64_t *toff;      // n+1
    uint32_t *tlog;      // n: log2 table capacity
    uint32_t *keys;      // T
    uint32_t *cnt;       // T
    uint32_t *ccount;    // occupied slots per compaction chunk (nch)
    uint64_t *cbase;     // nch+1: exclusive scan of ccount
    uint64_t nch;        // compaction chunks of the table arena
    uint64_t *qout;      // n+1: output offsets
    uint32_t *out_v;
    uint32_t *out_c;
    int load_shift;
};

__device__ __forceinline__ uint32_t log2_ceil(uint64_t x)
{
    return x <= 1 ? 0u : 64u - (uint32_t)__clzll((long long)(x - 1));
}

// Exclusive scans of walkers and table capacities, one CTA.
__global__ void __launch_bounds__(kPrepThreads) prep_kernel(BatchArgs a)
{
    const uint32_t n = *a.n_dev;
    __shared__ unsigned long long warp_w[kPrepThreads / 32], warp_t[kPrepThreads / 32];
    __shared__ unsigned long long carry_w, carry_t;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        carry_w = 0;
        carry_t = 0;
    }
    __syncthreads();
    for (uint32_t base = 0; base < n; base += kPrepThreads) {
        const uint32_t q = base + threadIdx.x;
        unsigned long long w = 0, t = 0;
        if (q < n) {
            w = a.walkers[q];
            const uint32_t lg = max(5u, log2_ceil(w << a.load_shift));
            a.tlog[q] = lg;
            t = 1ull << lg;
        }
        unsigned long long iw = w, it = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long xw = __shfl_up_sync(kFull, iw, o), xt = __shfl_up_sync(kFull, it, o);
            if (lane >= o) {
                iw += xw;
                it += xt;
            }
        }
        if (lane == 31) {
            warp_w[wid] = iw;
            warp_t[wid] = it;
        }
        __syncthreads();
        if (wid == 0) {
            unsigned long long sw = warp_w[lane], st = warp_t[lane];
            unsigned long long pw = sw, pt = st;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long xw = __shfl_up_sync(kFull, pw, o), xt = __shfl_up_sync(kFull, pt, o);
                if (lane >= o) {
                    pw += xw;
                    pt += xt;
                }
            }
            warp_w[lane] = pw - sw;
            warp_t[lane] = pt - st;
        }
        __syncthreads();
        if (q < n) {
            a.woff[q] = carry_w + warp_w[wid] + iw - w;
            a.toff[q] = carry_t + warp_t[wid] + it - t;
        }
        __syncthreads();
        if (threadIdx.x == kPrepThreads - 1) {
            carry_w += warp_w[wid] + iw;
            carry_t += warp_t[wid] + it;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.woff[n] = carry_w;
        a.toff[n] = carry_t;
        a.hdr->n = n;
        a.hdr->W = carry_w;
        a.hdr->T = carry_t;
        a.hdr->next = 0;
        a.hdr->error = 0;
        a.hdr->stats[0] = a.hdr->stats[1] = a.hdr->stats[2] = 0;
    }
}

__global__ void clear_kernel(BatchArgs a)
{
    const uint64_t T = a.hdr->T;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T; i += stride) {
        a.keys[i] = kEmpty;
        a.cnt[i] = 0;
    }
}

__device__ __forceinline__ void table_add(const BatchArgs &a, uint32_t q, uint32_t v)
{
    const uint64_t base = a.toff[q];
    const uint32_t lg = a.tlog[q];
    const uint64_t mask = (1ull << lg) - 1;
    uint64_t slot = ((uint64_t)(v * 0x9E3779B1u)) & mask;
    for (uint64_t probe = 0; probe <= mask; probe++) {
        uint32_t *k = &a.keys[base + slot];
        uint32_t cur = *(volatile uint32_t *)k;
        if (cur == kEmpty) cur = atomicCAS(k, kEmpty, v);
        if (cur == kEmpty || cur == v) {
            atomicAdd(&a.cnt[base + slot], 1u);
            return;
        }
        slot = (slot + 1) & mask;
    }
    atomicAdd(&a.hdr->error, 1ull);
}

__device__ __forceinline__ uint32_t find_query(const uint32_t *s_off, const uint64_t *g_off, bool in_smem, uint32_t n,
                                               uint64_t g)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        const uint64_t o = in_smem ? (uint64_t)s_off[mid] : g_off[mid];
        if (g < o)
            hi = mid - 1;
        else
            lo = mid;
    }
    return lo;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) batch_walk_kernel(BatchArgs a)
{
    extern __shared__ uint32_t s_off[];
    const uint32_t n = (uint32_t)a.hdr->n;
    const uint64_t W = a.hdr->W;
    const bool in_smem = n <= a.smem_queries && W < (1ull << 32);
    if (in_smem)
        for (uint32_t i = threadIdx.x; i < n; i += BLOCK) s_off[i] = (uint32_t)a.woff[i];
    __syncthreads();
    if (n == 0) return;

    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const uint64_t keep = l2_policy_evict_last(), stream = l2_policy_evict_first();
    uint32_t cur = 0, step = 0, q = 0;
    uint64_t idx = 0, seed = 0;
    bool active = false, exhausted = false;
    unsigned long long n_upd = 0, n_mov = 0;

    while (true) {
        const unsigned idle = __ballot_sync(kFull, !active);
        if (idle != 0u && !exhausted && (__popc(idle) >= kRefillMin || idle == kFull)) {
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&a.hdr->next, (unsigned long long)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if (base + __popc(idle) >= W) exhausted = true;
            if (!active) {
                const uint64_t g = base + __popc(idle & lt_mask);
                if (g < W) {
                    q = find_query(s_off, a.woff, in_smem, n, g);
                    idx = g - a.woff[q];
                    seed = a.seeds[q];
                    cur = a.src[q];
                    step = ppr_length(seed, 0, idx, a.thr);
                    active = true;
                }
            }
        }
        if (__ballot_sync(kFull, active) == 0u) {
            if (exhausted) break;
            continue;
        }
        if (!active) continue;
        // app/ppr.cu:22-42
        const uint32_t s = step;
        n_upd++;
        bool done = false;
        if (s == 1) {
            done = true;
        } else {
            step = s - 1;
            uint64_t first, deg;
            if (a.rowptr32) {
                const uint32_t f = ld_nc_u32(a.rowptr32 + cur, keep);
                first = f;
                deg = ld_nc_u32(a.rowptr32 + cur + 1, keep) - f;
            } else {
                first = ld_nc_u64(a.rowptr + cur, keep);
                deg = ld_nc_u64(a.rowptr + cur + 1, keep) - first;
            }
            if (deg > 0) {
                const Rand4 r = walk_draw(seed, s, kTagStep, 0, idx);
                cur = ld_nc_stream_u32(a.col + first + mod_u64(r64_of(r), deg), stream);
                n_mov++;
            } else {
                done = true;
            }
        }
        if (done) {
            table_add(a, q, cur);
            active = false;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_upd += __shfl_down_sync(kFull, n_upd, o);
        n_mov += __shfl_down_sync(kFull, n_mov, o);
    }
    if (lane == 0) {
        atomicAdd(&a.hdr->stats[0], n_upd);
        atomicAdd(&a.hdr->stats[1], n_mov);
    }
}

__device__ unsigned block_count(unsigned v, unsigned *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kRowThreads / 32; w++) t += sh[w];
    return t;
}

// Compaction in fixed chunks of the table arena, so that one large table
// (a Zipf-heavy query) is spread over many CTAs: count the occupied slots of
// every chunk, scan the counts, then every CTA writes its chunk's pairs in
// slot order; a query's output offset is the chunk base of its first slot
// plus the occupied slots between that chunk's start and the table.
constexpr uint64_t kCompactChunk = 4096;

__global__ void __launch_bounds__(kRowThreads) chunk_count_kernel(BatchArgs a)
{
    __shared__ unsigned sh[kRowThreads / 32];
    const uint64_t T = a.toff[(uint32_t)a.hdr->n];
    for (uint64_t c = blockIdx.x; c < a.nch; c += gridDim.x) {
        const uint64_t b = c * kCompactChunk, e = b + kCompactChunk < T ? b + kCompactChunk : T;
        unsigned cnt = 0;
        for (uint64_t i = b + threadIdx.x; i < e; i += kRowThreads) cnt += a.keys[i] != kEmpty;
        const unsigned t = block_count(cnt, sh);
        if (threadIdx.x == 0) a.ccount[c] = t;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kRowThreads) chunk_compact_kernel(BatchArgs a)
{
    __shared__ unsigned sh[kRowThreads / 32];
    const uint64_t T = a.toff[(uint32_t)a.hdr->n];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint64_t c = blockIdx.x; c < a.nch && c * kCompactChunk < T; c += gridDim.x) {
        const uint64_t b = c * kCompactChunk, e = b + kCompactChunk < T ? b + kCompactChunk : T;
        uint64_t base = a.cbase[c];
        for (uint64_t t0 = b; t0 < e; t0 += kRowThreads) {
            const uint64_t i = t0 + threadIdx.x;
            const bool occ = i < e && a.keys[i] != kEmpty;
            const unsigned m = __ballot_sync(kFull, occ);
            if (lane == 0) sh[wid] = __popc(m);
            __syncthreads();
            unsigned before = 0, total = 0;
            for (int w = 0; w < kRowThreads / 32; w++) {
                if (w < wid) before += sh[w];
                total += sh[w];
            }
            if (occ) {
                const uint64_t pos = base + before + __popc(m & ((1u << lane) - 1u));
                a.out_v[pos] = a.keys[i];
                a.out_c[pos] = a.cnt[i];
            }
            base += total;
            __syncthreads();
        }
    }
}

// One warp per query q (and q = n): qout[q] = occupied slots before toff[q].
__global__ void query_offsets_kernel(BatchArgs a)
{
    const uint32_t n = (uint32_t)a.hdr->n;
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const uint64_t nwarps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t q = warp; q <= n; q += nwarps) {
        const uint64_t s = a.toff[q], c = s / kCompactChunk;
        unsigned cnt = 0;
        for (uint64_t i = c * kCompactChunk + lane; i < s; i += 32) cnt += a.keys[i] != kEmpty;
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(kFull, cnt, o);
        if (lane == 0) a.qout[q] = a.cbase[c] + cnt;
    }
}

template <int BLOCK>
int walk_occupancy(size_t smem)
{
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_walk_kernel<BLOCK>, BLOCK, smem);
    return occ < 1 ? 1 : occ;
}

}  // namespace

struct BatchState {
    lt_engine *e = nullptr;
    uint32_t qcap = 0;
    uint64_t wcap = 0, tcap = 0;
    Header *d_hdr = nullptr;
    uint32_t *d_src = nullptr, *d_tlog = nullptr, *d_keys = nullptr, *d_cnt = nullptr, *d_ccount = nullptr;
    uint32_t *d_n = nullptr;
    uint64_t *d_walkers = nullptr, *d_seeds = nullptr, *d_woff = nullptr, *d_toff = nullptr, *d_qout = nullptr;
    uint64_t *d_scan_tmp = nullptr, *d_cbase = nullptr;
    uint64_t nch = 0;  // compaction chunks of the table arena
    uint32_t *d_out_v = nullptr, *d_out_c = nullptr;
    BatchTune tune;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t graph_thr = 0;
    BatchTune graph_tune;
    Header h_hdr{};
    uint32_t h_n = 0;
};

namespace {

void free_buffers(BatchState &b)
{
    for (void *p : {(void *)b.d_hdr, (void *)b.d_n, (void *)b.d_src, (void *)b.d_tlog, (void *)b.d_keys, (void *)b.d_cnt,
                    (void *)b.d_ccount, (void *)b.d_walkers, (void *)b.d_seeds, (void *)b.d_woff, (void *)b.d_toff,
                    (void *)b.d_qout, (void *)b.d_scan_tmp, (void *)b.d_cbase, (void *)b.d_out_v, (void *)b.d_out_c})
        if (p) cudaFree(p);
    b.d_hdr = nullptr;
    b.d_n = nullptr;
    b.d_src = b.d_tlog = b.d_keys = b.d_cnt = b.d_ccount = b.d_out_v = b.d_out_c = nullptr;
    b.d_walkers = b.d_seeds = b.d_woff = b.d_toff = b.d_qout = b.d_scan_tmp = b.d_cbase = nullptr;
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    b.exec = nullptr;
    b.graph = nullptr;
}

template <typename T>
lt_status dalloc(T **p, uint64_t count)
{
    if (cudaMalloc((void **)p, sizeof(T) * (count ? count : 1)) != cudaSuccess) {
        cudaGetLastError();
        return fail(LT_ERR_NOMEM, "cudaMalloc of %llu bytes failed", (unsigned long long)(sizeof(T) * count));
    }
    return LT_OK;
}

uint64_t table_slots(const uint64_t *walkers, uint32_t n, int shift)
{
    uint64_t t = 0;
    for (uint32_t q = 0; q < n; q++) {
        uint64_t c = 32;
        while (c < (walkers[q] << shift)) c <<= 1;
        t += c;
    }
    return t;
}

lt_status ensure(BatchState &b, uint32_t n, uint64_t W, uint64_t T)
{
    if (b.d_hdr && n <= b.qcap && W <= b.wcap && T <= b.tcap) return LT_OK;
    const uint32_t qcap = std::max<uint32_t>(n, std::max<uint32_t>(b.qcap, 64));
    const uint64_t wcap = std::max<uint64_t>(W, b.wcap);
    const uint64_t tcap = std::max<uint64_t>(T, b.tcap);
    free_buffers(b);
    b.qcap = qcap;
    b.wcap = wcap;
    b.tcap = tcap;
    LT_TRY(dalloc(&b.d_hdr, 1));
    LT_TRY(dalloc(&b.d_n, 1));
    LT_TRY(dalloc(&b.d_src, qcap));
    LT_TRY(dalloc(&b.d_tlog, qcap));
    b.nch = tcap / kCompactChunk + 1;
    LT_TRY(dalloc(&b.d_ccount, b.nch));
    LT_TRY(dalloc(&b.d_cbase, b.nch + 1));
    LT_TRY(dalloc(&b.d_walkers, qcap));
    LT_TRY(dalloc(&b.d_seeds, qcap));
    LT_TRY(dalloc(&b.d_woff, qcap + 1));
    LT_TRY(dalloc(&b.d_toff, qcap + 1));
    LT_TRY(dalloc(&b.d_qout, qcap + 1));
    LT_TRY(dalloc(&b.d_scan_tmp, scan_tmp_elems(b.nch)));
    LT_TRY(dalloc(&b.d_keys, tcap));
    LT_TRY(dalloc(&b.d_cnt, tcap));
    LT_TRY(dalloc(&b.d_out_v, wcap));
    LT_TRY(dalloc(&b.d_out_c, wcap));
    return LT_OK;
}

BatchArgs args_of(lt_engine *e, BatchState &b, uint64_t thr)
{
    BatchArgs a{};
    a.n_dev = b.d_n;
    a.smem_queries = std::min<uint32_t>(b.qcap, kSmemQueries);
    a.rowptr = e->d_rowptr;
    a.rowptr32 = e->d_rowptr32;
    a.col = e->d_col;
    a.V = e->g->V;
    a.thr = thr;
    a.hdr = b.d_hdr;
    a.src = b.d_src;
    a.walkers = b.d_walkers;
    a.seeds = b.d_seeds;
    a.woff = b.d_woff;
    a.toff = b.d_toff;
    a.tlog = b.d_tlog;
    a.keys = b.d_keys;
    a.cnt = b.d_cnt;
    a.ccount = b.d_ccount;
    a.cbase = b.d_cbase;
    a.nch = b.nch;
    a.qout = b.d_qout;
    a.out_v = b.d_out_v;
    a.out_c = b.d_out_c;
    a.load_shift = b.tune.load_shift;
    return a;
}

cudaError_t launch_walk(const BatchArgs &a, const BatchTune &t, int sms, cudaStream_t st)
{
    const size_t smem = 4ull * a.smem_queries;
    int occ = 1;
    switch (t.block) {
    case 128: occ = walk_occupancy<128>(smem); break;
    case 512: occ = walk_occupancy<512>(smem); break;
    default: occ = walk_occupancy<256>(smem); break;
    }
    if (t.ctas_per_sm > 0 && t.ctas_per_sm < occ) occ = t.ctas_per_sm;
    const int grid = sms * occ;
    switch (t.block) {
    case 128: batch_walk_kernel<128><<<grid, 128, smem, st>>>(a); break;
    case 512: batch_walk_kernel<512><<<grid, 512, smem, st>>>(a); break;
    default: batch_walk_kernel<256><<<grid, 256, smem, st>>>(a); break;
    }
    return cudaGetLastError();
}

// The batch pipeline on `st` for the queries already in the state's buffers
// (their count in d_n).
lt_status enqueue_pipeline(lt_engine *e, BatchState &b, uint64_t thr, cudaStream_t st)
{
    BatchArgs a = args_of(e, b, thr);
    prep_kernel<<<1, kPrepThreads, 0, st>>>(a);
    clear_kernel<<<e->sms * 8, 256, 0, st>>>(a);
    LT_CUDA_TRY(cudaGetLastError());
    LT_CUDA_TRY(launch_walk(a, b.tune, e->sms, st));
    const unsigned chunk_ctas = (unsigned)std::min<uint64_t>(b.nch, (uint64_t)e->sms * 16);
    chunk_count_kernel<<<chunk_ctas, kRowThreads, 0, st>>>(a);
    LT_CUDA_TRY(cudaGetLastError());
    LT_CUDA_TRY((exclusive_scan<uint32_t, uint64_t>(b.d_ccount, b.nch, b.d_cbase, b.d_scan_tmp, st)));
    chunk_compact_kernel<<<chunk_ctas, kRowThreads, 0, st>>>(a);
    const unsigned qblocks = (unsigned)std::min<uint64_t>(((uint64_t)b.qcap + 1) * 32 / 256 + 1, (uint64_t)e->sms * 16);
    query_offsets_kernel<<<qblocks, 256, 0, st>>>(a);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

// Replay the captured pipeline (capturing it first when the buffers, the
// stop probability or the tuning changed); n goes to the device first.
lt_status run_graph(lt_engine *e, BatchState &b, uint32_t n, uint64_t thr, cudaStream_t st)
{
    b.h_n = n;
    LT_CUDA_TRY(cudaMemcpyAsync(b.d_n, &b.h_n, 4, cudaMemcpyHostToDevice, st));
    const bool stale = !b.exec || b.graph_thr != thr || b.graph_tune.block != b.tune.block ||
                       b.graph_tune.ctas_per_sm != b.tune.ctas_per_sm || b.graph_tune.load_shift != b.tune.load_shift;
    if (stale) {
        if (b.exec) cudaGraphExecDestroy(b.exec);
        if (b.graph) cudaGraphDestroy(b.graph);
        b.exec = nullptr;
        b.graph = nullptr;
        cudaStream_t cap;
        LT_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        LT_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        const lt_status s = enqueue_pipeline(e, b, thr, cap);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (s != LT_OK) return s;
        LT_CUDA_TRY(ce);
        b.graph = g;
        LT_CUDA_TRY(cudaGraphInstantiate(&b.exec, b.graph, 0));
        b.graph_thr = thr;
        b.graph_tune = b.tune;
    }
    LT_CUDA_TRY(cudaGraphLaunch(b.exec, st));
    return LT_OK;
}

lt_status check_inputs(lt_engine *e, uint32_t n, float prob)
{
    if (!e->resident || !e->d_rowptr)
        return fail(LT_ERR_UNSUPPORTED, "batched PPR needs every partition cached on the device");
    if (!(prob > 0.0f && prob <= 1.0f)) return fail(LT_ERR_INVALID, "PPR stop probability must be in (0, 1]");
    if (n == 0) return fail(LT_ERR_INVALID, "empty batch");
    LT_CUDA_TRY(cudaSetDevice(e->device));
    return engine_ensure_loaded(e);
}

}  // namespace

lt_status batch_create(lt_engine *e, BatchState **out)
{
    BatchState *b = new BatchState();
    b->e = e;
    *out = b;
    return LT_OK;
}

void batch_destroy(BatchState *b)
{
    if (!b) return;
    free_buffers(*b);
    delete b;
}

BatchTune batch_tune(const lt_engine *e) { return e->batch ? e->batch->tune : BatchTune{}; }

lt_status batch_run_device(lt_engine *e, uint32_t n, const uint32_t *d_sources, const uint64_t *d_walkers,
                           const uint64_t *d_seeds, float prob, uint64_t *d_offsets, uint32_t *d_vertices,
                           uint32_t *d_counts, uint64_t out_capacity, cudaStream_t st)
{
    LT_TRY(check_inputs(e, n, prob));
    LT_CUDA_TRY(cudaSetDevice(e->device));
    if (!e->batch) LT_TRY(batch_create(e, &e->batch));
    BatchState &b = *e->batch;
    // the walker total and table size are needed on the host to size buffers
    std::vector<uint64_t> w(n);
    LT_CUDA_TRY(cudaMemcpyAsync(w.data(), d_walkers, 8ull * n, cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaStreamSynchronize(st));
    uint64_t W = 0;
    for (uint64_t x : w) W += x;
    if (W > out_capacity) return fail(LT_ERR_CAPACITY, "output capacity %llu is below the %llu walkers of the batch",
                                      (unsigned long long)out_capacity, (unsigned long long)W);
    LT_TRY(ensure(b, n, W, table_slots(w.data(), n, b.tune.load_shift)));
    LT_CUDA_TRY(cudaMemcpyAsync(b.d_src, d_sources, 4ull * n, cudaMemcpyDeviceToDevice, st));
    LT_CUDA_TRY(cudaMemcpyAsync(b.d_walkers, d_walkers, 8ull * n, cudaMemcpyDeviceToDevice, st));
    LT_CUDA_TRY(cudaMemcpyAsync(b.d_seeds, d_seeds, 8ull * n, cudaMemcpyDeviceToDevice, st));
    LT_TRY(run_graph(e, b, n, threshold53(prob), st));
    LT_CUDA_TRY(cudaMemcpyAsync(d_offsets, b.d_qout, 8ull * (n + 1), cudaMemcpyDeviceToDevice, st));
    LT_CUDA_TRY(cudaMemcpyAsync(d_vertices, b.d_out_v, 4ull * W, cudaMemcpyDeviceToDevice, st));
    LT_CUDA_TRY(cudaMemcpyAsync(d_counts, b.d_out_c, 4ull * W, cudaMemcpyDeviceToDevice, st));
    return LT_OK;
}

lt_status batch_run(lt_engine *e, uint32_t n, const uint32_t *sources, const uint64_t *walkers, const uint64_t *seeds,
                    float prob, uint64_t *out_offsets, uint32_t *out_vertices, uint32_t *out_counts,
                    uint64_t out_capacity)
{
    LT_TRY(check_inputs(e, n, prob));
    for (uint32_t q = 0; q < n; q++)
        if (sources[q] >= e->g->V) return fail(LT_ERR_INVALID, "query %u: source %u out of range", q, sources[q]);
    LT_CUDA_TRY(cudaSetDevice(e->device));
    if (!e->batch) LT_TRY(batch_create(e, &e->batch));
    BatchState &b = *e->batch;
    uint64_t W = 0;
    for (uint32_t q = 0; q < n; q++) W += walkers[q];
    if (W > out_capacity) return fail(LT_ERR_CAPACITY, "output capacity %llu is below the %llu walkers of the batch",
                                      (unsigned long long)out_capacity, (unsigned long long)W);
    LT_TRY(ensure(b, n, W, table_slots(walkers, n, b.tune.load_shift)));
    cudaStream_t st = e->s_compute;
    const double t0 = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
    LT_CUDA_TRY(cudaMemcpyAsync(b.d_src, sources, 4ull * n, cudaMemcpyHostToDevice, st));
    LT_CUDA_TRY(cudaMemcpyAsync(b.d_walkers, walkers, 8ull * n, cudaMemcpyHostToDevice, st));
    if (seeds) {
        LT_CUDA_TRY(cudaMemcpyAsync(b.d_seeds, seeds, 8ull * n, cudaMemcpyHostToDevice, st));
    } else {
        std::vector<uint64_t> s(n, e->cfg.seed);
        LT_CUDA_TRY(cudaMemcpy(b.d_seeds, s.data(), 8ull * n, cudaMemcpyHostToDevice));
    }
    LT_CUDA_TRY(cudaEventRecord(e->ev_k0, st));
    LT_TRY(run_graph(e, b, n, threshold53(prob), st));
    LT_CUDA_TRY(cudaEventRecord(e->ev_k1, st));
    LT_CUDA_TRY(cudaMemcpyAsync(&b.h_hdr, b.d_hdr, sizeof(Header), cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaMemcpyAsync(out_offsets, b.d_qout, 8ull * (n + 1), cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaStreamSynchronize(st));
    const uint64_t total = out_offsets[n];
    LT_CUDA_TRY(cudaMemcpyAsync(out_vertices, b.d_out_v, 4ull * total, cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaMemcpyAsync(out_counts, b.d_out_c, 4ull * total, cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaStreamSynchronize(st));
    if (b.h_hdr.error) return fail(LT_ERR_CAPACITY, "a per-query table overflowed");
    float ms = 0;
    cudaEventElapsedTime(&ms, e->ev_k0, e->ev_k1);
    e->stats = lt_stats{};
    e->stats.updates = b.h_hdr.stats[0];
    e->stats.moves = b.h_hdr.stats[1];
    e->stats.step_kernel_ms = ms;
    e->stats.computing_ms = ms;
    e->stats.computing_calls = 1;
    e->stats.iterations = 1;
    e->stats.kernel_launches = 6;
    e->stats.running_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count() - t0;
    return LT_OK;
}

// Autotuner: times the pipeline on a synthetic batch (512 queries of 4096
// walkers from evenly spread sources) for each block size and table load
// factor and keeps the fastest.
lt_status batch_autotune(lt_engine *e)
{
    if (!e->resident) return fail(LT_ERR_UNSUPPORTED, "batched PPR needs every partition cached on the device");
    LT_CUDA_TRY(cudaSetDevice(e->device));
    if (!e->batch) LT_TRY(batch_create(e, &e->batch));
    BatchState &b = *e->batch;
    const uint32_t n = 512;
    std::vector<uint32_t> src(n);
    std::vector<uint64_t> w(n, 4096), seeds(n);
    for (uint32_t q = 0; q < n; q++) {
        src[q] = (uint32_t)(((uint64_t)q * 2654435761ull) % e->g->V);
        seeds[q] = 0x7u + q;
    }
    const uint64_t W = (uint64_t)n * 4096;
    std::vector<uint64_t> off(n + 1);
    std::vector<uint32_t> ov(W), oc(W);
    BatchTune best = b.tune;
    double best_ms = 1e30;
    for (int shift : {1, 2}) {
        for (int block : {128, 256, 512}) {
            b.tune.block = block;
            b.tune.load_shift = shift;
            b.tune.ctas_per_sm = 0;
            double ms_min = 1e30;
            for (int rep = 0; rep < 3; rep++) {
                LT_TRY(batch_run(e, n, src.data(), w.data(), seeds.data(), 0.15f, off.data(), ov.data(), oc.data(), W));
                ms_min = std::min(ms_min, e->stats.step_kernel_ms);
            }
            if (ms_min < best_ms) {
                best_ms = ms_min;
                best = b.tune;
            }
        }
    }
    b.tune = best;
    b.tune.tuned = true;
    return LT_OK;
}

}  // namespace lt
