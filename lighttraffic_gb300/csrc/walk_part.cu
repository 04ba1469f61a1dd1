// walk_part.cu -- step kernel for partially cached graphs and the bucketing
// (scatter) kernel.
//
// Replaces randomWalkInsidePool[AllBatch] / randomWalkOutsidePool and the
// insertToQueue kernels (src/WalkManager.h:60-282) together with the 1-thread
// page kernels of src/buffer/Pool.h:484-528.
//
// Step kernel (persistent, one walker per lane, warp-aggregated refill):
//   input  = the chunks queued for one partition, plus walkers created lazily
//            from their ordinal (PPR source walkers, per-vertex starts);
//   a walker keeps stepping while the partition holding its vertex is readable
//   -- cached in a device slot, or mapped from pinned host memory for a
//   zero-copy pass -- which generalises the reference's "walk while inside the
//   partition" (src/WalkManager.h:239-240) to every cached partition;
//   updates that read no graph data (the final PPR / PageRank count, PageRank
//   teleports) run wherever the walker is;
//   a walker whose next update needs an unreadable partition is written to a
//   staging area (warp-aggregated slot reservation) and counted in a
//   per-destination histogram (shared memory, flushed once per CTA).
// Scatter kernel: appends staged walkers to their destination queues; a CTA
// counts its tile per destination in shared memory and reserves one range per
// destination with one global atomic (the two-level scheme of
// src/WalkManager.h:122-190), into chunks the host allocated beforehand.
#include <algorithm>

#include "lt_core.cuh"
#include "mem.cuh"
#include "scan.cuh"
#include "walk_part.h"

namespace lt {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
// idle lanes a warp waits for before refilling them (all lanes: always): the
// refill sits on the warp's critical path and PPR's geometric walk lengths
// would otherwise trigger one nearly every iteration (also in zero-copy
// launches, where refills are short beside host reads: on c2, thresholds 8
// and 2 there made runs 4 % and 6 % slower)
constexpr int kRefillMin = 24;

__device__ __forceinline__ uint32_t find_part(const uint32_t *off, uint32_t P, uint32_t v)
{
    uint32_t lo = 0, hi = P - 1;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (v < off[mid])
            hi = mid - 1;
        else
            lo = mid;
    }
    return lo;
}

// Row offsets stay in L2 (evict-last), column entries stream (evict-first).
__device__ __forceinline__ uint64_t ld_u64(unsigned long long addr, uint64_t keep)
{
    return ld_nc_u64(reinterpret_cast<const void *>(addr), keep);
}
__device__ __forceinline__ uint32_t ld_u32(unsigned long long addr, uint64_t stream)
{
    return ld_nc_stream_u32(reinterpret_cast<const void *>(addr), stream);
}

// Row of vertex cur in the lane's readable partition [nb, ne): the address of
// its first column entry and its degree.  Row offsets are u64 global edge
// offsets (rowptr slices in the slots, the reference's layout), or, with the
// compact device-resident index (a.rp32), u32 offsets relative to the
// partition's first edge; eb is then the partition's edge count, which ends
// the last vertex's row.
// hot: the vertex carries the tier mark (compact index only).
__device__ __forceinline__ void row_at(bool rp32, unsigned long long rp, unsigned long long col, uint64_t eb,
                                       uint32_t cur, uint32_t nb, uint32_t ne, uint64_t keep,
                                       unsigned long long &first_addr, uint64_t &deg, bool &hot)
{
    const uint32_t rel = cur - nb;
    if (rp32) {
        const uint32_t lo_m = ld_nc_u32(reinterpret_cast<const void *>(rp + 4ull * rel), keep);
        const uint32_t hi = cur + 1 < ne
                                ? ld_nc_u32(reinterpret_cast<const void *>(rp + 4ull * (rel + 1)), keep) & ~kHotMark
                                : (uint32_t)eb;
        const uint32_t lo = lo_m & ~kHotMark;
        first_addr = col + 4ull * lo;
        deg = hi - lo;
        hot = (lo_m & kHotMark) != 0;
    } else {
        hot = false;
        const uint64_t first = ld_u64(rp + 8ull * rel, keep);
        deg = ld_u64(rp + 8ull * (rel + 1), keep) - first;
        first_addr = col + 4ull * (first - eb);
    }
}

// Address of the first column entry of marked vertex v in the tier.
__device__ __forceinline__ unsigned long long hot_first(const StepArgs &a, uint32_t v, uint64_t keep)
{
    const uint2 w = ld_nc_u2(a.hot_words + (v >> 5), keep);
    const uint32_t rank = w.y + __popc(w.x & ((1u << (v & 31)) - 1u));
    return (unsigned long long)(a.hot_pool + ld_nc_u32(a.hot_off + rank, keep));
}

// Row of the next update in the lane's readable range; a marked vertex of a
// zero-copy partition is read from the tier instead of host memory.
template <bool HOT>
__device__ __forceinline__ void row_of(const StepArgs &a, unsigned long long rp, unsigned long long col, uint64_t eb,
                                       uint32_t cur, uint32_t nb, uint32_t ne, bool zc, uint64_t keep,
                                       unsigned long long &first_addr, uint64_t &deg, bool &zc_read)
{
    bool marked;
    row_at(a.rp32, rp, col, eb, cur, nb, ne, keep, first_addr, deg, marked);
    zc_read = zc;
    if (HOT && marked && zc) {
        first_addr = hot_first(a, cur, keep);
        zc_read = false;
    }
}

// A PPR walk ends at v: count it (single run) or add it to the query's table
// (linear probing, u32 counts) and mark one more walker of the query done.
__device__ __forceinline__ void ppr_count(const StepArgs &a, uint32_t qs, uint32_t v)
{
    if (!a.q_seed) {
        red_add1_u64((unsigned long long *)&a.counts[v], l2_policy_evict_last());
        return;
    }
    const uint64_t base = a.q_toff[qs];
    const uint64_t mask = (1ull << a.q_tlog[qs]) - 1;
    uint64_t slot = ((uint64_t)(v * 0x9E3779B1u)) & mask;
    bool added = false;
    for (uint64_t probe = 0; probe <= mask && !added; probe++) {
        uint32_t *k = &a.q_keys[base + slot];
        uint32_t old = *(volatile uint32_t *)k;
        if (old == 0xFFFFFFFFu) old = atomicCAS(k, 0xFFFFFFFFu, v);
        if (old == 0xFFFFFFFFu || old == v) {
            atomicAdd(&a.q_cnt[base + slot], 1u);
            added = true;
        }
        slot = (slot + 1) & mask;
    }
    if (!added) atomicAdd(a.q_error, 1ull);
    __threadfence();
    atomicAdd(&a.q_done[qs], 1ull);
}

// Resident CTAs per SM the register budget is sized for: PPR fits 48
// registers with no spills (5 x 256 threads), PageRank and generic walks 40
// (6 x 256); unbounded, PPR took 55 (4 CTAs) and hops in flight were the limit
// on zero-copy reads.
template <int APP>
constexpr int part_min_blocks() { return APP == kPPR ? 5 : 6; }

// HOT: the hot-vertex tier is on (a.hot_on); a separate instance, so that
// runs without the tier keep the registers of the kernel without it.
template <int APP, bool HOT>
__global__ void __launch_bounds__(kPartBlock, part_min_blocks<APP>()) walk_part_kernel(StepArgs a)
{
    extern __shared__ uint32_t smem[];
    const uint32_t P = a.t.P;
    const bool in_smem = P <= kSmemPartMax;
    uint32_t *s_off = smem;
    uint32_t *s_hist = smem + (P + 1);
    uint32_t *s_visit = s_hist + P;
    uint32_t *s_zc = s_visit + P;
    if (in_smem) {
        for (uint32_t i = threadIdx.x; i <= P; i += blockDim.x) s_off[i] = a.t.node_off[i];
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
            s_hist[i] = 0;
            s_visit[i] = 0;
        }
        for (uint32_t i = threadIdx.x; i < (P + 31) / 32; i += blockDim.x) s_zc[i] = a.zc_mask[i];
    }
    __syncthreads();
    const uint32_t *off = in_smem ? s_off : a.t.node_off;
    uint32_t *hist = in_smem ? s_hist : a.hist;
    uint32_t *visit = in_smem ? s_visit : a.visits;

    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const uint64_t total = a.n_chunk_walkers + a.lazy_count;
    const uint64_t keep = l2_policy_evict_last(), stream = l2_policy_evict_first();

    uint32_t cur = 0, step = 0, idx = 0, hop = 0, qs = 0;
    uint64_t seed = a.seed;
    bool active = false, exhausted = false;
    // cached readable partition of the lane
    uint32_t cp_nb = 1, cp_ne = 0;
    unsigned long long cp_rp = 0, cp_col = 0;
    uint64_t cp_eb = 0;
    bool cp_zc = false;
    // per-thread statistics of this launch (a launch makes far fewer than
    // 2^32 updates per thread); widened in the warp reduction at the end
    uint32_t n_upd = 0, n_mov = 0, n_tel = 0, n_zc = 0, n_exit = 0, n_fin = 0;

    while (true) {
        const unsigned idle = __ballot_sync(kFull, !active);
        if (idle != 0u && !exhausted && (__popc(idle) >= kRefillMin || idle == kFull)) {
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.next, (unsigned long long)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if (base + __popc(idle) >= total) exhausted = true;
            if (!active) {
                const uint64_t my = base + __popc(idle & lt_mask);
                if (my < a.n_chunk_walkers) {
                    uint32_t wi, j;
                    if (!a.work_off) {
                        wi = (uint32_t)(my / kChunk);
                        j = (uint32_t)(my % kChunk);
                    } else {
                        uint32_t lo = 0, hi = a.n_work - 1;
                        while (lo < hi) {
                            const uint32_t mid = lo + (hi - lo + 1) / 2;
                            if (my < a.work_off[mid])
                                hi = mid - 1;
                            else
                                lo = mid;
                        }
                        wi = lo;
                        j = (uint32_t)(my - a.work_off[lo]);
                    }
                    const uint32_t k = a.work_chunks[wi];
                    const uint32_t *c = reinterpret_cast<const uint32_t *>(a.arena + (uint64_t)k * kChunkBytes);
                    cur = c[j];
                    step = c[kChunk + j];
                    idx = c[2 * kChunk + j];
                    qs = c[3 * kChunk + j];
                    // A walker taken from a queue chunk was counted as
                    // entering its partition when it was staged there; the
                    // empty range (2, 1) forces its lookup and marks it as
                    // not a new entry (counting it again would rank uncached
                    // partitions by the walkers that queued at them, i.e.
                    // by the cache state).  (1, 0) is the plain empty range.
                    cp_nb = 2;
                    cp_ne = 1;
                    if (a.q_seed) seed = a.q_seed[qs];
                    active = true;
                } else if (my < total) {
                    const uint64_t t = a.lazy_begin + (my - a.n_chunk_walkers);
                    if (a.lazy_mode == kStartPerVertex) {
                        idx = (uint32_t)per_vertex_id(t, a.lazy_nb, a.lazy_n, a.V);
                        cur = a.lazy_nb + (uint32_t)(t % a.lazy_n);
                    } else {
                        idx = (uint32_t)t;
                        cur = start_vertex(a.lazy_mode, a.source, a.V, a.seed, a.run, idx);
                    }
                    qs = 0;
                    seed = a.seed;
                    step = APP == kPPR ? ppr_length(a.seed, a.run, idx, a.thr) : a.length;
                    if (APP == kWalk && a.paths) a.paths[(uint64_t)idx * (a.length + 1)] = cur;
                    active = true;
                }
                hop = a.length - step;
            }
        }
        if (__ballot_sync(kFull, active) == 0u) {
            if (exhausted) break;
            continue;
        }

        // Does the next update read the graph, and is the walker's partition readable?
        Rand4 r{};
        bool need_graph = false, emit = false;
        uint32_t dest = 0;
        if (active) {
            if (APP == kPPR) {
                need_graph = step >= 2;
            } else if (APP == kPageRank) {
                if (step >= 2) {
                    r = walk_draw(seed, step, kTagStep, a.run, idx);
                    need_graph = m53_of(r) < a.thr;
                }
            } else {
                need_graph = true;
            }
            if (need_graph && (cur < cp_nb || cur >= cp_ne)) {
                const uint32_t p = find_part(off, P, cur);
                if (!(cp_nb == 2 && cp_ne == 1)) atomicAdd(&visit[p], 1u);
                unsigned long long rp, col = 0;
                if (p == a.zc_part) {
                    rp = a.zc_rp | 1ull;
                    col = a.zc_col;
                } else {
                    rp = *(volatile const unsigned long long *)&a.t.rp_addr[p];
                    if (rp != 0ull) {
                        col = *(volatile const unsigned long long *)&a.t.col_addr[p];
                    } else if (in_smem && ((s_zc[p >> 5] >> (p & 31)) & 1u)) {
                        rp = (a.zc_rp_base + (a.rp32 ? 4ull : 8ull) * off[p]) | 1ull;
                        col = a.zc_col_base + 4ull * a.t.edge_off[p];
                    }
                }
                bool hot = false;
                if (HOT && rp == 0ull) {
                    // unreadable partition: a marked vertex is read from the
                    // tier, as a one-vertex readable range of the lane
                    const uint32_t lo_m = ld_nc_u32(reinterpret_cast<const void *>(a.zc_rp_base + 4ull * cur), keep);
                    if (lo_m & kHotMark) {
                        const uint32_t lo = lo_m & ~kHotMark;
                        cp_eb = cur + 1 < off[p + 1]
                                    ? ld_nc_u32(reinterpret_cast<const void *>(a.zc_rp_base + 4ull * (cur + 1)), keep) &
                                          ~kHotMark
                                    : a.t.edge_off[p + 1] - a.t.edge_off[p];
                        cp_nb = cur;
                        cp_ne = cur + 1;
                        cp_rp = a.zc_rp_base + 4ull * cur;
                        cp_col = hot_first(a, cur, keep) - 4ull * lo;
                        cp_zc = false;
                        hot = true;
                    }
                }
                if (hot) {
                } else if (rp == 0ull) {
                    emit = true;
                    dest = p;
                    cp_nb = 1;
                    cp_ne = 0;
                } else {
                    cp_nb = off[p];
                    cp_ne = off[p + 1];
                    cp_rp = rp & ~1ull;
                    cp_col = col;
                    cp_eb = a.rp32 ? a.t.edge_off[p + 1] - a.t.edge_off[p] : a.t.edge_off[p];
                    cp_zc = (rp & 1ull) != 0;
                }
            }
        }
        const unsigned em = __ballot_sync(kFull, emit);
        if (em != 0u) {
            const int leader = __ffs(em) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.out_n, (unsigned long long)__popc(em));
            base = __shfl_sync(kFull, base, leader);
            if (emit) {
                const uint64_t pos = base + __popc(em & lt_mask);
                a.out_cur[pos] = cur;
                a.out_step[pos] = step;
                a.out_idx[pos] = idx;
                a.out_dest[pos] = dest;
                a.out_q[pos] = qs;
                atomicAdd(&hist[dest], 1u);
                active = false;
                n_exit++;
            }
        }
        if (!active) continue;

        const uint32_t s = step;
        n_upd++;
        bool done = false;
        if (APP == kPPR) {
            // app/ppr.cu:22-42
            if (s == 1) {
                ppr_count(a, qs, cur);
                done = true;
            } else {
                step = s - 1;
                unsigned long long fa;
                uint64_t deg;
                bool zc_read;
                row_of<HOT>(a, cp_rp, cp_col, cp_eb, cur, cp_nb, cp_ne, cp_zc, keep, fa, deg, zc_read);
                if (deg > 0) {
                    const Rand4 q = walk_draw(seed, s, kTagStep, a.run, idx);
                    cur = ld_u32(fa + 4ull * mod_u64(r64_of(q), deg), stream);
                    n_mov++;
                    n_zc += zc_read;
                } else {
                    ppr_count(a, qs, cur);
                    done = true;
                }
            }
        } else if (APP == kPageRank) {
            // app/pagerank.cu:26-44; a vertex without out-edges teleports.
            red_add1_u64((unsigned long long *)&a.counts[cur], keep);
            if (s == 1) {
                done = true;
            } else {
                step = s - 1;
                const uint64_t r64 = r64_of(r);
                bool tele = !need_graph;
                if (!tele) {
                    unsigned long long fa;
                    uint64_t deg;
                    bool zc_read;
                    row_of<HOT>(a, cp_rp, cp_col, cp_eb, cur, cp_nb, cp_ne, cp_zc, keep, fa, deg, zc_read);
                    if (deg > 0) {
                        cur = ld_u32(fa + 4ull * mod_u64(r64, deg), stream);
                        n_mov++;
                        n_zc += zc_read;
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
            unsigned long long fa;
            uint64_t deg;
            bool zc_read;
            row_of<HOT>(a, cp_rp, cp_col, cp_eb, cur, cp_nb, cp_ne, cp_zc, keep, fa, deg, zc_read);
            uint32_t *path = a.paths ? a.paths + (uint64_t)idx * (a.length + 1) : nullptr;
            if (deg > 0) {
                const Rand4 q = walk_draw(seed, s, kTagStep, a.run, idx);
                cur = ld_u32(fa + 4ull * mod_u64(r64_of(q), deg), stream);
                n_mov++;
                n_zc += zc_read;
                hop++;
                if (path) path[hop] = cur;
                step = s - 1;
            } else {
                if (path)
                    for (uint32_t h = hop + 1; h <= a.length; h++) path[h] = kInvalidNode;
                step = 0;
            }
            done = step == 0;
        }
        if (done) {
            active = false;
            n_fin++;
            if (a.endpoints) a.endpoints[idx] = cur;
        }
    }

    uint64_t w_upd = n_upd, w_mov = n_mov, w_tel = n_tel, w_zc = n_zc, w_exit = n_exit, w_fin = n_fin;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        w_upd += __shfl_down_sync(kFull, w_upd, o);
        w_mov += __shfl_down_sync(kFull, w_mov, o);
        w_tel += __shfl_down_sync(kFull, w_tel, o);
        w_zc += __shfl_down_sync(kFull, w_zc, o);
        w_exit += __shfl_down_sync(kFull, w_exit, o);
        w_fin += __shfl_down_sync(kFull, w_fin, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stats[0], (unsigned long long)w_upd);
        atomicAdd(&a.stats[1], (unsigned long long)w_mov);
        atomicAdd(&a.stats[2], (unsigned long long)w_tel);
        atomicAdd(&a.stats[3], (unsigned long long)w_zc);
        atomicAdd(&a.stats[4], (unsigned long long)w_exit);
        atomicAdd(&a.stats[5], (unsigned long long)w_fin);
    }
    if (in_smem) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
            if (s_hist[i]) atomicAdd(&a.hist[i], s_hist[i]);
            if (s_visit[i]) atomicAdd(&a.visits[i], s_visit[i]);
        }
    }
}

// Tile of kScatterItems walkers per thread.
constexpr int kScatterItems = 4;

__global__ void __launch_bounds__(kPartBlock) scatter_kernel(ScatterArgs a)
{
    extern __shared__ uint32_t smem[];
    const uint32_t P = a.P;
    const bool in_smem = P <= kSmemPartMax;
    uint32_t *s_cnt = smem;       // P: walkers of this tile per destination
    uint32_t *s_base = smem + P;  // P: reserved base slot per destination
    const uint64_t tile = (uint64_t)kPartBlock * kScatterItems;
    for (uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < a.n; t0 += (uint64_t)gridDim.x * tile) {
        uint32_t rank[kScatterItems], dest[kScatterItems];
        if (in_smem) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) s_cnt[i] = 0;
            __syncthreads();
        }
#pragma unroll
        for (int k = 0; k < kScatterItems; k++) {
            const uint64_t i = t0 + (uint64_t)k * kPartBlock + threadIdx.x;
            dest[k] = 0xFFFFFFFFu;
            if (i < a.n) {
                dest[k] = a.in_dest[i];
                rank[k] = in_smem ? atomicAdd(&s_cnt[dest[k]], 1u) : atomicAdd(&a.cursor[dest[k]], 1u);
            }
        }
        if (in_smem) {
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x)
                if (s_cnt[i]) s_base[i] = atomicAdd(&a.cursor[i], s_cnt[i]);
            __syncthreads();
        }
#pragma unroll
        for (int k = 0; k < kScatterItems; k++) {
            const uint64_t i = t0 + (uint64_t)k * kPartBlock + threadIdx.x;
            if (i < a.n) {
                const uint32_t d = dest[k];
                const uint32_t pos = in_smem ? s_base[d] + rank[k] : rank[k];
                const uint32_t chunk = a.plan_chunks[a.win_off[d] + pos / kChunk];
                uint32_t *c = reinterpret_cast<uint32_t *>(a.arena + (uint64_t)chunk * kChunkBytes);
                const uint32_t j = pos % kChunk;
                c[j] = a.in_cur[i];
                c[kChunk + j] = a.in_step[i];
                c[2 * kChunk + j] = a.in_idx[i];
                c[3 * kChunk + j] = a.in_q[i];
            }
        }
        if (in_smem) __syncthreads();
    }
}

// Bucketing by a block-local counting sort (P <= kSmemPartMax).  A tile of
// T = BLOCK x ITEMS staged walkers is ranked per destination in shared
// memory (shared atomics), the per-destination counts are scanned across the
// block and reserved in the destination windows with one global atomic per
// (tile, destination) -- the two-level scheme of insertToQueueKernel
// (src/WalkManager.h:122-190) -- and the tile is written back through its
// sort permutation as per-destination runs: consecutive threads write
// consecutive queue slots.
//
// The CTAs are persistent and double-buffered: while a tile is sorted, the
// bulk-copy unit (cp.async.bulk, one copy per field, completion counted on an
// mbarrier) brings the CTA's next tile from the staging area into shared
// memory, so the kernel issues no global loads of walker fields.  A tile's
// chunk ids are looked up once per destination, not per walker.  The staged
// field arrays start 16-byte aligned and hold n rounded up to 4 words (the
// copies round up to 16 bytes).  If a copy does not complete within a second,
// the CTA records it in *err and reads the remaining tiles from global memory
// directly, so no walker is lost.
// Two shapes, chosen by the autotuner: 1024 threads x 4 walkers (T = 4096,
// the default; one CTA per SM) and 512 threads x 4 walkers (T = 2048; two
// CTAs per SM, so that one CTA's barrier waits overlap the other's work; on
// c2 its bucketing took 145 ms per run against 97).  Every phase of a tile
// ends at a block barrier; 256-thread CTAs of a 4096-walker tile left 8
// warps per SM to hide the latencies (c2s launch: 46 against 38 us).
constexpr int kBucketFields = 5;                    // cur, step, idx, query, dest
constexpr uint64_t kBulkWaitNs = 1000000000ull;     // bounded wait on one tile's copies

template <int BLOCK, int ITEMS>
size_t bucket_smem(uint32_t P)
{
    const uint64_t T = (uint64_t)BLOCK * ITEMS;
    // two tiles of kBucketFields u32 fields | 2 mbarriers | 4 u32 per destination | u16 permutation
    return 4 * 2 * kBucketFields * T + 16 + 16ull * P + 2 * T;
}

template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) bucket_sort_kernel(ScatterArgs a)
{
    constexpr uint32_t T = BLOCK * ITEMS;
    constexpr uint32_t kPerMax = kSmemPartMax / BLOCK;
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint32_t warp_tot[BLOCK / 32];
    __shared__ uint32_t tile_total;
    const uint32_t P = a.P;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + 2 * kBucketFields * T);
    uint32_t *s_off = reinterpret_cast<uint32_t *>(mbar + 2);  // P: tile count, then offset in the sorted tile
    uint32_t *s_base = s_off + P;                              // P: first reserved slot of the window
    uint32_t *s_ch0 = s_base + P;                              // P: chunk holding s_base
    uint32_t *s_ch1 = s_ch0 + P;                               // P: the next chunk, where the run crosses into it
    uint16_t *s_inv = reinterpret_cast<uint16_t *>(s_ch1 + P); // T: tile position at sorted position j
    const uint32_t *src[kBucketFields] = {a.in_cur, a.in_step, a.in_idx, a.in_q, a.in_dest};
    if (a.err && (*(volatile unsigned int *)a.err & 2u)) return;
    const uint64_t n = a.n_dev ? *a.n_dev : a.n;
    const uint64_t tiles = (n + T - 1) / T;
    bool bulk = true;
#pragma unroll
    for (int f = 0; f < kBucketFields; f++) bulk = bulk && ((uintptr_t)src[f] & 15) == 0;
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    // thread 0: copies of tile `tile` into buffer b
    auto issue = [&](uint64_t tile, int b) {
        const uint64_t t0 = tile * T;
        const uint32_t m = (uint32_t)(n - t0 < T ? n - t0 : T);
        const uint32_t bytes = (4 * m + 15) & ~15u;
        mbar_arrive_expect_tx(&mbar[b], kBucketFields * bytes);
#pragma unroll
        for (int f = 0; f < kBucketFields; f++) bulk_load_smem(smem + (b * kBucketFields + f) * T, src[f] + t0, bytes, &mbar[b]);
    };
    // copies issued into / completions waited for on buffer 0 and buffer 1
    uint32_t issued0 = 0, issued1 = 0, waited0 = 0, waited1 = 0;
    uint64_t tile = blockIdx.x;
    if (bulk && tile < tiles) {
        if (threadIdx.x == 0) issue(tile, 0);
        issued0++;
    }
    const uint32_t per = (P + BLOCK - 1) / BLOCK;  // destinations a thread reserves and scans
    for (uint32_t it = 0; tile < tiles; tile += gridDim.x, it++) {
        const int b = it & 1;
        const uint64_t t0 = tile * T;
        const uint32_t m = (uint32_t)(n - t0 < T ? n - t0 : T);
        if (bulk && tile + gridDim.x < tiles) {
            // buffer b^1 was last read by the previous tile, which ended at a barrier
            if (threadIdx.x == 0) issue(tile + gridDim.x, b ^ 1);
            if (b) issued0++;
            else issued1++;
        }
        for (uint32_t i = threadIdx.x; i < P; i += BLOCK) s_off[i] = 0;
        if (bulk) {
            const bool ok = mbar_wait_bounded(&mbar[b], (b ? waited1 : waited0) & 1, kBulkWaitNs);
            if (ok) {
                if (b) waited1++;
                else waited0++;
            }
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0 && a.err) atomicOr(a.err, 1u);
                bulk = false;
            }
        } else {
            __syncthreads();
        }
        const uint32_t *f_cur, *f_step, *f_idx, *f_q, *f_dest;
        if (bulk) {
            const uint32_t *buf = smem + b * kBucketFields * T;
            f_cur = buf, f_step = buf + T, f_idx = buf + 2 * T, f_q = buf + 3 * T, f_dest = buf + 4 * T;
        } else {
            f_cur = a.in_cur + t0, f_step = a.in_step + t0, f_idx = a.in_idx + t0, f_q = a.in_q + t0,
            f_dest = a.in_dest + t0;
        }
        uint32_t dest[ITEMS], rank[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            const uint32_t i = k * BLOCK + threadIdx.x;
            dest[k] = i < m ? f_dest[i] : 0xFFFFFFFFu;
            rank[k] = dest[k] != 0xFFFFFFFFu ? atomicAdd(&s_off[dest[k]], 1u) : 0u;
        }
        __syncthreads();
        // reserve each destination's run: window starts and atomics first,
        // then the chunk lookups that depend on both
        uint32_t cnt[kPerMax], base[kPerMax], win[kPerMax];
        uint32_t mine = 0;
#pragma unroll
        for (uint32_t j = 0; j < kPerMax; j++) {
            const uint32_t d = threadIdx.x * per + j;
            cnt[j] = j < per && d < P ? s_off[d] : 0;
            win[j] = cnt[j] ? a.win_off[d] : 0;
        }
#pragma unroll
        for (uint32_t j = 0; j < kPerMax; j++) {
            const uint32_t d = threadIdx.x * per + j;
            base[j] = cnt[j] ? atomicAdd(&a.cursor[d], cnt[j]) : 0;
            mine += cnt[j];
        }
#pragma unroll
        for (uint32_t j = 0; j < kPerMax; j++) {
            if (!cnt[j]) continue;
            const uint32_t d = threadIdx.x * per + j;
            const uint32_t w = win[j] + base[j] / kChunk;
            s_base[d] = base[j];
            s_ch0[d] = a.plan_chunks[w];
            // a run (at most T < kChunk walkers) spans one chunk or two
            s_ch1[d] = (base[j] + cnt[j] - 1) / kChunk != base[j] / kChunk ? a.plan_chunks[w + 1] : 0u;
        }
        uint32_t off = scan_detail::block_exclusive<uint32_t, BLOCK>(mine, warp_tot, &tile_total);
#pragma unroll
        for (uint32_t j = 0; j < kPerMax; j++) {
            const uint32_t d = threadIdx.x * per + j;
            if (j < per && d < P) {
                s_off[d] = off;
                off += cnt[j];
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < ITEMS; k++)
            if (dest[k] != 0xFFFFFFFFu) s_inv[s_off[dest[k]] + rank[k]] = (uint16_t)(k * BLOCK + threadIdx.x);
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < m; j += BLOCK) {
            const uint32_t i = s_inv[j];
            const uint32_t d = f_dest[i];
            const uint32_t b0 = s_base[d];
            const uint32_t g = b0 + (j - s_off[d]);
            const uint32_t chunk = g / kChunk == b0 / kChunk ? s_ch0[d] : s_ch1[d];
            uint32_t *c = reinterpret_cast<uint32_t *>(a.arena + (uint64_t)chunk * kChunkBytes);
            const uint32_t jj = g % kChunk;
            c[jj] = f_cur[i];
            c[kChunk + jj] = f_step[i];
            c[2 * kChunk + jj] = f_idx[i];
            c[3 * kChunk + jj] = f_q[i];
        }
        __syncthreads();
    }
    // copies still in flight exist only after a wait gave up: wait for them
    // (bounded) before this CTA's shared memory is released
    while (waited0 < issued0 && mbar_wait_bounded(&mbar[0], waited0 & 1, kBulkWaitNs)) waited0++;
    while (waited1 < issued1 && mbar_wait_bounded(&mbar[1], waited1 & 1, kBulkWaitNs)) waited1++;
}

// One CTA plans every destination: per destination the chunks its arrivals
// need (new ones and, with an open tail chunk, that one), two block scans for
// the stack and window positions, then the windows in destination order.
constexpr int kPlanBlock = 1024;

__global__ void __launch_bounds__(kPlanBlock) plan_kernel(PlanArgs a)
{
    constexpr uint32_t kPerMax = kSmemPartMax / kPlanBlock;
    __shared__ uint32_t warp_tot[kPlanBlock / 32];
    __shared__ uint32_t tot_new, tot_slots;
    const uint32_t P = a.P;
    const uint32_t per = (P + kPlanBlock - 1) / kPlanBlock;
    uint32_t h[kPerMax], fill[kPerMax], tail[kPerMax], nnew[kPerMax];
    uint32_t my_new = 0, my_slots = 0;
#pragma unroll
    for (uint32_t j = 0; j < kPerMax; j++) {
        const uint32_t d = threadIdx.x * per + j;
        h[j] = j < per && d < P ? a.hist[d] : 0;
        fill[j] = 0;
        tail[j] = kNoChunk;
        nnew[j] = 0;
        if (h[j]) {
            const uint32_t tc = a.tail_chunk[d], tf = a.tail_fill[d];
            const bool open = tc != kNoChunk && tf < kChunk;
            fill[j] = open ? tf : 0;
            tail[j] = open ? tc : kNoChunk;
            const uint32_t chunks = (uint32_t)(((uint64_t)fill[j] + h[j] + kChunk - 1) / kChunk);
            nnew[j] = chunks - (open ? 1u : 0u);
            my_new += nnew[j];
            my_slots += chunks;
        }
    }
    uint32_t pos_new = scan_detail::block_exclusive<uint32_t, kPlanBlock>(my_new, warp_tot, &tot_new);
    uint32_t pos_slot = scan_detail::block_exclusive<uint32_t, kPlanBlock>(my_slots, warp_tot, &tot_slots);
    if (tot_new > a.n_stack || tot_slots > a.plan_cap) {
        if (threadIdx.x == 0 && a.err) atomicOr(a.err, 2u);
        return;
    }
#pragma unroll
    for (uint32_t j = 0; j < kPerMax; j++) {
        const uint32_t d = threadIdx.x * per + j;
        if (j >= per || d >= P) continue;
        a.cursor[d] = fill[j];
        a.win_off[d] = h[j] ? pos_slot : 0;
        if (!h[j]) continue;
        if (tail[j] != kNoChunk) a.plan_chunks[pos_slot++] = tail[j];
        for (uint32_t c = 0; c < nnew[j]; c++) a.plan_chunks[pos_slot++] = a.stack[pos_new++];
    }
}

__global__ void inject_kernel(InjectArgs a)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const uint64_t pos = a.cursor + i;
        const uint32_t chunk = a.plan_chunks[pos / kChunk];
        uint32_t *c = reinterpret_cast<uint32_t *>(a.arena + (uint64_t)chunk * kChunkBytes);
        const uint32_t j = (uint32_t)(pos % kChunk);
        c[j] = a.source;
        c[kChunk + j] = ppr_length(a.seed, 0, i, a.thr);
        c[2 * kChunk + j] = (uint32_t)i;
        c[3 * kChunk + j] = a.qslot;
    }
}

template <int APP>
int occ_part(size_t smem)
{
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(walk_part_kernel<APP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(walk_part_kernel<APP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, walk_part_kernel<APP, false>, kPartBlock, smem);
    return n;
}

}  // namespace

size_t part_smem(uint32_t P) { return P <= kSmemPartMax ? sizeof(uint32_t) * (3ull * P + 1 + (P + 31) / 32) : 0; }

int part_grid(int app, int /*start*/, int device, size_t smem, int ctas_per_sm)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int occ = app == kPPR ? occ_part<kPPR>(smem) : app == kPageRank ? occ_part<kPageRank>(smem) : occ_part<kWalk>(smem);
    if (ctas_per_sm > 0 && ctas_per_sm < occ) occ = ctas_per_sm;
    if (occ < 1) occ = 1;
    return sms * occ;
}

cudaError_t launch_walk_part(const StepArgs &a, int app, int grid, cudaStream_t st)
{
    const size_t smem = part_smem(a.t.P);
    switch (app) {
    case kPPR:
        if (a.hot_on)
            walk_part_kernel<kPPR, true><<<grid, kPartBlock, smem, st>>>(a);
        else
            walk_part_kernel<kPPR, false><<<grid, kPartBlock, smem, st>>>(a);
        break;
    case kPageRank:
        if (a.hot_on)
            walk_part_kernel<kPageRank, true><<<grid, kPartBlock, smem, st>>>(a);
        else
            walk_part_kernel<kPageRank, false><<<grid, kPartBlock, smem, st>>>(a);
        break;
    default:
        if (a.hot_on)
            walk_part_kernel<kWalk, true><<<grid, kPartBlock, smem, st>>>(a);
        else
            walk_part_kernel<kWalk, false><<<grid, kPartBlock, smem, st>>>(a);
        break;
    }
    return cudaGetLastError();
}

cudaError_t launch_plan(const PlanArgs &a, cudaStream_t st)
{
    if (a.P > kSmemPartMax) return cudaErrorInvalidValue;
    plan_kernel<<<1, kPlanBlock, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_inject(const InjectArgs &a, int device, cudaStream_t st)
{
    if (a.n == 0) return cudaSuccess;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint64_t blocks = (a.n + 255) / 256;
    if (blocks > (uint64_t)sms * 4) blocks = (uint64_t)sms * 4;
    inject_kernel<<<(unsigned)blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_scatter(const ScatterArgs &a, int device, cudaStream_t st)
{
    if (a.n == 0) return cudaSuccess;
    // per device and partition count: SMs, and the CTAs per SM of both shapes
    // (one launch per wave iteration: no attribute queries on that path)
    static thread_local int cached_device = -1;
    static thread_local uint32_t cached_P = 0;
    static thread_local int sms = 0, smem_optin = 0, per_sm_big = 0, per_sm_small = 0;
    if (cached_device != device || (a.P <= kSmemPartMax && cached_P != a.P)) {
        cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
        // room for the kernels' static shared memory
        const int dyn = smem_optin - 1024;
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(bucket_sort_kernel<1024, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(bucket_sort_kernel<512, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
        per_sm_big = per_sm_small = 0;
        if (e == cudaSuccess && a.P <= kSmemPartMax && bucket_smem<1024, 4>(a.P) + 1024 <= (size_t)smem_optin)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_big, bucket_sort_kernel<1024, 4>, 1024,
                                                              bucket_smem<1024, 4>(a.P));
        if (e == cudaSuccess && a.P <= kSmemPartMax)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_small, bucket_sort_kernel<512, 4>, 512,
                                                              bucket_smem<512, 4>(a.P));
        if (e != cudaSuccess) {
            cached_device = -1;
            return e;
        }
        cached_device = device;
        cached_P = a.P;
    }
    if (a.P <= kSmemPartMax) {
        // 4096-walker tiles unless 2048 are asked for (items 8), or where
        // 4096 do not fit (P above about 3 700)
        const bool small = a.items == 8 || per_sm_big == 0;
        const int block = small ? 512 : 1024;
        const size_t smem = small ? bucket_smem<512, 4>(a.P) : bucket_smem<1024, 4>(a.P);
        const uint64_t tile = (uint64_t)block * 4;
        const uint64_t tiles = (a.n + tile - 1) / tile;
        const int per_sm = std::max(1, small ? per_sm_small : per_sm_big);
        const uint64_t blocks = std::min<uint64_t>(tiles, (uint64_t)sms * per_sm);
        if (small)
            bucket_sort_kernel<512, 4><<<(unsigned)blocks, block, smem, st>>>(a);
        else
            bucket_sort_kernel<1024, 4><<<(unsigned)blocks, block, smem, st>>>(a);
        return cudaGetLastError();
    }
    const uint64_t tile = (uint64_t)kPartBlock * kScatterItems;
    uint64_t blocks = (a.n + tile - 1) / tile;
    const uint64_t cap = (uint64_t)sms * 8;
    if (blocks > cap) blocks = cap;
    const size_t smem = a.P <= kSmemPartMax ? sizeof(uint32_t) * 2ull * a.P : 0;
    scatter_kernel<<<(unsigned)blocks, kPartBlock, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace lt
