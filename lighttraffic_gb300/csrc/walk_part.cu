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
// would otherwise trigger one nearly every iteration
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
__device__ __forceinline__ void row_at(bool rp32, unsigned long long rp, unsigned long long col, uint64_t eb,
                                       uint32_t cur, uint32_t nb, uint32_t ne, uint64_t keep,
                                       unsigned long long &first_addr, uint64_t &deg)
{
    const uint32_t rel = cur - nb;
    if (rp32) {
        const uint32_t lo = ld_nc_u32(reinterpret_cast<const void *>(rp + 4ull * rel), keep);
        const uint32_t hi =
            cur + 1 < ne ? ld_nc_u32(reinterpret_cast<const void *>(rp + 4ull * (rel + 1)), keep) : (uint32_t)eb;
        first_addr = col + 4ull * lo;
        deg = hi - lo;
    } else {
        const uint64_t first = ld_u64(rp + 8ull * rel, keep);
        deg = ld_u64(rp + 8ull * (rel + 1), keep) - first;
        first_addr = col + 4ull * (first - eb);
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

template <int APP>
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
                if (rp == 0ull) {
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
                row_at(a.rp32, cp_rp, cp_col, cp_eb, cur, cp_nb, cp_ne, keep, fa, deg);
                if (deg > 0) {
                    const Rand4 q = walk_draw(seed, s, kTagStep, a.run, idx);
                    cur = ld_u32(fa + 4ull * mod_u64(r64_of(q), deg), stream);
                    n_mov++;
                    n_zc += cp_zc;
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
                    row_at(a.rp32, cp_rp, cp_col, cp_eb, cur, cp_nb, cp_ne, keep, fa, deg);
                    if (deg > 0) {
                        cur = ld_u32(fa + 4ull * mod_u64(r64, deg), stream);
                        n_mov++;
                        n_zc += cp_zc;
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
            row_at(a.rp32, cp_rp, cp_col, cp_eb, cur, cp_nb, cp_ne, keep, fa, deg);
            uint32_t *path = a.paths ? a.paths + (uint64_t)idx * (a.length + 1) : nullptr;
            if (deg > 0) {
                const Rand4 q = walk_draw(seed, s, kTagStep, a.run, idx);
                cur = ld_u32(fa + 4ull * mod_u64(r64_of(q), deg), stream);
                n_mov++;
                n_zc += cp_zc;
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
// kBucketTile staged walkers is ranked per destination in shared memory
// (shared atomics), the per-destination counts are scanned across the block
// and reserved in the destination windows with one global atomic per
// (tile, destination) -- the two-level scheme of insertToQueueKernel
// (src/WalkManager.h:122-190) -- and the walkers are laid out sorted by
// destination in shared memory, so that the write-back is a sequence of
// per-destination runs: consecutive threads write consecutive queue slots.
// The plain scatter above wrote each walker with four isolated 4-byte stores
// and made one global atomic per (1024-walker tile, destination), i.e.
// nearly one per walker when the walkers spread over ~1000 partitions.
// The tile is kPartBlock x ITEMS walkers (ITEMS 16: 4096, the default; 8:
// 2048, chosen by the autotuner when it is faster).
constexpr int kBucketFields = 5;  // cur, step, idx, query, dest

template <int ITEMS>
size_t bucket_smem(uint32_t P)
{
    return sizeof(uint32_t) * (2ull * P + (uint64_t)kBucketFields * kPartBlock * ITEMS);
}

template <int ITEMS>
__global__ void __launch_bounds__(kPartBlock, 2) bucket_sort_kernel(ScatterArgs a)
{
    constexpr int kBucketItems = ITEMS;
    constexpr int kBucketTile = kPartBlock * ITEMS;
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t warp_tot[kPartBlock / 32];
    __shared__ uint32_t tile_total;
    const uint32_t P = a.P;
    uint32_t *s_cnt = smem;       // P: walkers of the tile per destination, then their offsets in the sorted tile
    uint32_t *s_base = smem + P;  // P: first reserved slot of the destination's window
    uint32_t *s_cur = s_base + P;
    uint32_t *s_step = s_cur + kBucketTile;
    uint32_t *s_idx = s_step + kBucketTile;
    uint32_t *s_q = s_idx + kBucketTile;
    uint32_t *s_dest = s_q + kBucketTile;
    const uint32_t per = (P + kPartBlock - 1) / kPartBlock;  // destinations a thread reserves and scans
    for (uint64_t t0 = (uint64_t)blockIdx.x * kBucketTile; t0 < a.n; t0 += (uint64_t)gridDim.x * kBucketTile) {
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) s_cnt[i] = 0;
        __syncthreads();
        uint32_t dest[kBucketItems], rank[kBucketItems];
#pragma unroll
        for (int k = 0; k < kBucketItems; k++) {
            const uint64_t i = t0 + (uint64_t)k * kPartBlock + threadIdx.x;
            dest[k] = i < a.n ? a.in_dest[i] : 0xFFFFFFFFu;
            rank[k] = dest[k] != 0xFFFFFFFFu ? atomicAdd(&s_cnt[dest[k]], 1u) : 0u;
        }
        __syncthreads();
        uint32_t mine = 0;
        for (uint32_t j = 0; j < per; j++) {
            const uint32_t d = threadIdx.x * per + j;
            if (d < P) {
                const uint32_t c = s_cnt[d];
                if (c) s_base[d] = atomicAdd(&a.cursor[d], c);
                mine += c;
            }
        }
        uint32_t off = scan_detail::block_exclusive<uint32_t>(mine, warp_tot, &tile_total);
        for (uint32_t j = 0; j < per; j++) {
            const uint32_t d = threadIdx.x * per + j;
            if (d < P) {
                const uint32_t c = s_cnt[d];
                s_cnt[d] = off;
                off += c;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kBucketItems; k++) {
            if (dest[k] == 0xFFFFFFFFu) continue;
            const uint64_t i = t0 + (uint64_t)k * kPartBlock + threadIdx.x;
            const uint32_t pos = s_cnt[dest[k]] + rank[k];
            s_cur[pos] = a.in_cur[i];
            s_step[pos] = a.in_step[i];
            s_idx[pos] = a.in_idx[i];
            s_q[pos] = a.in_q[i];
            s_dest[pos] = dest[k];
        }
        __syncthreads();
        const uint32_t m = (uint32_t)min((uint64_t)kBucketTile, a.n - t0);
        for (uint32_t j = threadIdx.x; j < m; j += blockDim.x) {
            const uint32_t d = s_dest[j];
            const uint32_t g = s_base[d] + (j - s_cnt[d]);
            const uint32_t chunk = a.plan_chunks[a.win_off[d] + g / kChunk];
            uint32_t *c = reinterpret_cast<uint32_t *>(a.arena + (uint64_t)chunk * kChunkBytes);
            const uint32_t jj = g % kChunk;
            c[jj] = s_cur[j];
            c[kChunk + jj] = s_step[j];
            c[2 * kChunk + jj] = s_idx[j];
            c[3 * kChunk + jj] = s_q[j];
        }
        __syncthreads();
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
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(walk_part_kernel<APP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, walk_part_kernel<APP>, kPartBlock, smem);
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
    case kPPR: walk_part_kernel<kPPR><<<grid, kPartBlock, smem, st>>>(a); break;
    case kPageRank: walk_part_kernel<kPageRank><<<grid, kPartBlock, smem, st>>>(a); break;
    default: walk_part_kernel<kWalk><<<grid, kPartBlock, smem, st>>>(a); break;
    }
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
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (a.P <= kSmemPartMax) {
        static thread_local int configured_device = -1;
        if (configured_device != device) {
            cudaError_t e = cudaFuncSetAttribute(bucket_sort_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)bucket_smem<16>(kSmemPartMax));
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(bucket_sort_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bucket_smem<8>(kSmemPartMax));
            if (e != cudaSuccess) return e;
            configured_device = device;
        }
        const int items = a.items == 8 ? 8 : 16;
        const size_t smem = items == 8 ? bucket_smem<8>(a.P) : bucket_smem<16>(a.P);
        const uint64_t tile = (uint64_t)kPartBlock * items;
        const uint64_t tiles = (a.n + tile - 1) / tile;
        const uint64_t per_sm = smem <= 72 * 1024 ? 3 : smem <= 110 * 1024 ? 2 : 1;
        const uint64_t blocks = std::min<uint64_t>(tiles, (uint64_t)sms * per_sm);
        if (items == 8)
            bucket_sort_kernel<8><<<(unsigned)blocks, kPartBlock, smem, st>>>(a);
        else
            bucket_sort_kernel<16><<<(unsigned)blocks, kPartBlock, smem, st>>>(a);
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
