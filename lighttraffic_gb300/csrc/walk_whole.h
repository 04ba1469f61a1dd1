// walk_whole.h -- launcher of the resident-graph step kernel.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lt {

constexpr int kWholeBlock = 256;

struct WholeArgs {
    const uint64_t *rowptr;  // u64[V+1], global edge offsets
    const uint32_t *col;     // u32[E]
    uint32_t V;
    uint32_t source;
    uint64_t W;              // walkers in this pass
    uint32_t length;         // PageRank / walk length
    uint32_t run;            // epoch index (random stream selector)
    uint64_t seed;
    uint64_t thr;            // floor(p 2^53): PPR stop prob or PageRank alpha
    uint64_t *counts;        // u64[V] or null (walk app)
    uint32_t *endpoints;     // u32[W] or null
    uint32_t *paths;         // u32[W*(length+1)] or null (walk app)
    uint64_t *next;          // scratch: next walker index (zeroed before launch)
    uint64_t *stats;         // u64[3] or null: updates, moves, teleports
    // Compact layout (launch with compact = true): u32 row offsets (E < 2^32)
    // and u32 counters (fewer than 2^32 counter updates in the launch)
    // replace rowptr and counts.  Half the bytes for the two arrays every
    // update reuses, so that they stay in L2 against the column stream.
    const uint32_t *rowptr32;
    uint32_t *counts32;
    // Packed layout (launch with layout kLayoutPacked): rows[2v] = first edge
    // of v (u32), rows[2v+1] = v's counter (u32).  The row offsets an update
    // reads and the counter it increments share one 32-byte sector.
    uint32_t *rows;
};

enum Layout : int { kLayoutWide = 0, kLayoutCompact = 1, kLayoutPacked = 2 };

// Persistent grid size: SMs x resident CTAs (capped by ctas_per_sm when > 0).
int whole_grid(int app, int start, int device, int ctas_per_sm, int layout = kLayoutWide);
cudaError_t launch_walk_whole(const WholeArgs &a, int app, int start, int grid, cudaStream_t st,
                              int layout = kLayoutWide);

}  // namespace lt
