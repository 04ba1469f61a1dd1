// batch.h -- batched multi-source PPR on a graph resident in HBM.
//
// Many PPR queries (source, walkers, seed) run in one persistent launch.
// Query q's walkers are ordinals [woff[q], woff[q+1]) of one index space; a
// walker's random stream is keyed by the query's seed and its index inside
// the query, so a query gives the same counts alone or in any batch, and the
// same counts as lt_run_ppr with that seed.  Endpoint counts (u32) are
// aggregated in per-query open-addressing hash tables and compacted into a
// per-query sparse output (vertex, count), grouped by query; the order of
// pairs inside a query is unspecified.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.h"

struct lt_engine;

namespace lt {

struct BatchTune {
    int block = 256;       // threads per CTA of the walk kernel
    int ctas_per_sm = 0;   // 0 = occupancy maximum
    int load_shift = 1;    // table capacity = next_pow2(walkers << load_shift)
    bool tuned = false;
};

struct BatchState;
lt_status batch_create(lt_engine *e, BatchState **out);
void batch_destroy(BatchState *b);

// Host inputs / outputs.  out_offsets: n+1 entries; out_vertices / out_counts:
// out_capacity entries (the sum of walkers always suffices).
lt_status batch_run(lt_engine *e, uint32_t n, const uint32_t *sources, const uint64_t *walkers,
                    const uint64_t *seeds, float prob, uint64_t *out_offsets, uint32_t *out_vertices,
                    uint32_t *out_counts, uint64_t out_capacity);

// Device inputs / outputs on `stream`; returns without waiting.
lt_status batch_run_device(lt_engine *e, uint32_t n, const uint32_t *d_sources, const uint64_t *d_walkers,
                           const uint64_t *d_seeds, float prob, uint64_t *d_offsets, uint32_t *d_vertices,
                           uint32_t *d_counts, uint64_t out_capacity, cudaStream_t stream);

lt_status batch_autotune(lt_engine *e);
BatchTune batch_tune(const lt_engine *e);

}  // namespace lt
