// walk_part.h -- out-of-core step and bucketing kernels.
//
// Walkers wait in per-partition queues made of fixed-size chunks.  A chunk is
// one contiguous block of kChunk walkers in structure-of-arrays form:
//     u32 cur[kChunk] | u32 step[kChunk] | u32 idx[kChunk] | u32 query[kChunk]
// so a chunk moves between device and host with a single copy.  Every chunk of
// a queue is full except its last one.  `query` is the walker's query slot
// when the engine serves many PPR queries at once (0 otherwise).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lt {

constexpr uint32_t kChunk = 8192;                         // walkers per chunk
constexpr uint64_t kChunkBytes = 16ull * kChunk;           // 128 KiB
constexpr int kPartBlock = 256;
constexpr uint32_t kSmemPartMax = 4096;                    // P up to this keeps node_off / histograms in smem
constexpr uint32_t kZcMaskWords = kSmemPartMax / 32;       // zero-copy set of one launch, one bit per partition

// Device view of the partition table: node / edge ranges of every partition
// and, for readable partitions, the addresses of their rowptr slice (n+1
// global edge offsets) and col slice -- a device cache slot, or pinned host
// memory read zero-copy, marked by bit 0 of the rowptr address.  An entry may
// change while a step kernel runs only from unreadable or zero-copy to a
// cache slot whose copy has completed; a slot is never overwritten while a
// kernel that may read it runs.
struct PartTable {
    const uint32_t *node_off;             // P+1
    const uint64_t *edge_off;             // P+1
    const unsigned long long *rp_addr;    // P, 0 = not readable
    const unsigned long long *col_addr;   // P
    uint32_t P;
};

struct StepArgs {
    PartTable t;
    uint8_t *arena;                // chunk arena
    const uint32_t *work_chunks;   // chunk ids of the partitions being drained
    uint64_t n_chunk_walkers;      // walkers in those chunks
    // null: one partition's chunks, all full except the last; otherwise the
    // first walker ordinal of each of the n_work chunks (chunks of several
    // partitions, each partition's last one partly filled)
    const uint64_t *work_off;
    uint32_t n_work;
    uint64_t lazy_begin;           // first lazy ordinal to create
    uint64_t lazy_count;           // lazy walkers to create in this pass
    uint32_t lazy_nb, lazy_n;      // per-vertex starts: vertex range [lazy_nb, lazy_nb + lazy_n)
    int lazy_mode;                 // lt::Start of the lazy walkers
    uint64_t W;                    // walkers of the run (per-vertex ordinal mapping)
    uint32_t V;
    uint32_t source;
    uint32_t length;
    uint32_t run;
    uint64_t seed;
    uint64_t thr;
    uint64_t *counts;
    uint32_t *endpoints;
    uint32_t *paths;
    // outputs for walkers that leave the readable partitions
    uint32_t *out_cur, *out_step, *out_idx, *out_dest;
    unsigned long long *out_n;     // staged walkers (atomic)
    uint32_t *hist;                // P: staged walkers per destination
    uint32_t *visits;              // P: walkers entering each partition (readable or not)
    unsigned long long *next;      // scratch: next input ordinal
    unsigned long long *stats;     // 8: updates, moves, teleports, zc moves, exits, finished, -, -
    // partition read zero-copy in this launch (0xFFFFFFFF = none) and its
    // device-visible addresses of pinned host memory
    uint32_t zc_part;
    unsigned long long zc_rp, zc_col;
    // further partitions read zero-copy in this launch (wave runs): bit p of
    // zc_mask (P <= kSmemPartMax only), read at zc_rp_base + 8 node_off[p]
    // (4 node_off[p] with rp32)
    // and zc_col_base + 4 edge_off[p] when the table marks p unreadable
    unsigned long long zc_rp_base, zc_col_base;
    uint32_t zc_mask[kZcMaskWords];
    // row offsets of every readable partition are u32 offsets relative to
    // the partition's first edge (the compact device-resident vertex index);
    // 0: u64 global edge offsets
    int rp32;
    // hot-vertex tier (hot_on, rp32 only): bit 31 of a vertex's entry in the
    // device index marks it as held in the tier; hot_words[v / 32] = {the
    // marks of vertices 32 (v / 32) .. + 31, tier rank of the first marked
    // one}, hot_off[rank] = word offset of its adjacency in hot_pool.  A hop
    // at a marked vertex of a partition outside the device cache reads its
    // column entry from hot_pool instead of host memory (or of waiting for
    // the partition).  Every reader of the index masks the mark.
    int hot_on;
    const uint2 *hot_words;
    const uint32_t *hot_off;
    const uint32_t *hot_pool;
    // query mode (serving many PPR queries): per query slot its key, table and
    // finished-walker counter; endpoints go to the query's table instead of
    // `counts`.  q_seed == null: single-run mode.
    uint32_t *out_q;
    const uint64_t *q_seed;
    const uint64_t *q_toff;
    const uint32_t *q_tlog;
    uint32_t *q_keys, *q_cnt;
    unsigned long long *q_done;
    unsigned long long *q_error;
};

struct ScatterArgs {
    const uint32_t *in_cur, *in_step, *in_idx, *in_dest, *in_q;
    uint64_t n;
    uint8_t *arena;
    uint32_t *cursor;              // P: next free slot offset in the destination's chunk window
    const uint32_t *win_off;       // P: start of the destination's window in plan_chunks
    const uint32_t *plan_chunks;   // chunk ids of every window
    uint32_t P;
    int items;                     // bucketing tile: 16 (0) = 4096 walkers, 8 = 2048
    unsigned int *err;             // bit 0 set when a tile's bulk copy did not complete in time;
                                   // the pass does nothing while bit 1 (a failed device plan) is set
    // non-null: the staged count lives here (device memory) and n only bounds it
    const unsigned long long *n_dev;
};

// Device-side plan of one bucketing pass, made right after the step kernel
// from its histogram so that no host round trip separates the two: the
// arrivals of destination d (hist[d]) go after the walkers of its open tail
// chunk, then into new chunks popped from the free stack in destination
// order.  The host replays the same arithmetic afterwards for its own queue
// bookkeeping.
struct PlanArgs {
    const uint32_t *hist;        // P: arrivals per destination
    const uint32_t *tail_chunk;  // P: last device chunk of d's queue, 0xFFFFFFFF = none
    const uint32_t *tail_fill;   // P: walkers in it
    const uint32_t *stack;       // free chunks, the next one to pop first
    uint32_t n_stack;
    uint32_t P;
    uint32_t *cursor, *win_off, *plan_chunks;  // the ScatterArgs plan
    uint64_t plan_cap;
    unsigned int *err;           // bit 1 set when the stack or the plan buffer is too small
};
constexpr uint32_t kNoChunk = 0xFFFFFFFFu;
constexpr uint32_t kHotMark = 0x80000000u;   // tier mark in a device index entry

// Walkers of newly admitted queries: walker i of query slot q (i < n) goes to
// position cursor + i of the chunk window, with PPR length from (seed, i).
struct InjectArgs {
    uint8_t *arena;
    const uint32_t *plan_chunks;
    uint32_t cursor;
    uint64_t n;
    uint32_t source, qslot;
    uint64_t seed, thr;
};

// Step-kernel grid: SMs x resident CTAs (capped at ctas_per_sm when > 0).
int part_grid(int app, int start, int device, size_t smem, int ctas_per_sm);
cudaError_t launch_inject(const InjectArgs &a, int device, cudaStream_t st);
size_t part_smem(uint32_t P);
cudaError_t launch_walk_part(const StepArgs &a, int app, int grid, cudaStream_t st);
cudaError_t launch_scatter(const ScatterArgs &a, int device, cudaStream_t st);
// P <= kSmemPartMax
cudaError_t launch_plan(const PlanArgs &a, cudaStream_t st);

// Ordinal t of the lazily created walkers of partition [nb, ne) under the
// per-vertex start: walkers j*V + v (v in [nb, ne)), ordered j-major.
__host__ __device__ inline uint64_t per_vertex_id(uint64_t t, uint32_t nb, uint32_t n, uint32_t V)
{
    return (t / n) * (uint64_t)V + nb + (t % n);
}

}  // namespace lt
