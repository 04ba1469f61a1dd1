// engine.h -- the engine object behind lt_engine_*.
#pragma once

#include <chrono>
#include <cstdint>
#include <vector>

#include "common.h"
#include "graph.h"
#include "batch.h"
#include "ooc.h"

namespace lt {
lt_status generate_rmat(int device, uint32_t scale, uint64_t E, double a, double b, double c, double d, uint64_t seed,
                        lt_graph &g);
}

struct lt_engine {
    lt_graph *g = nullptr;
    lt_engine_cfg cfg{};
    int device = 0;
    int sms = 0;
    cudaStream_t s_compute = nullptr, s_copy = nullptr, s_copyback = nullptr;
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;

    // Resident mode: every partition is cached and the partitions are laid out
    // back to back, which makes the cache one contiguous CSR.
    bool resident = false;
    uint64_t *d_rowptr = nullptr;
    uint32_t *d_col = nullptr;
    bool loaded = false;
    // compact layout (E < 2^32): u32 row offsets, and u32 counters for calls
    // whose counter updates stay below 2^32, widened to d_counts at the end
    uint32_t *d_rowptr32 = nullptr;
    uint32_t *d_counts32 = nullptr;

    uint64_t *d_counts = nullptr;  // u64[V]
    void *d_scratch = nullptr;     // lt_walk_scratch_bytes()
    uint64_t *d_stats = nullptr;   // u64[3]
    uint32_t *d_endpoints = nullptr;
    uint64_t endpoints_cap = 0;
    uint32_t *d_paths = nullptr;
    uint64_t paths_cap = 0;

    lt::Ooc *ooc = nullptr;          // out-of-core state when not every partition is cached
    lt::BatchState *batch = nullptr;  // batched multi-source PPR buffers and captured graph

    lt_stats stats{};
    lt_ooc_tune ooc_tune{};  // what lt_engine_autotune chose for the out-of-core engine
};

namespace lt {
lt_status engine_create(lt_graph *g, const lt_engine_cfg &cfg, lt_engine **out);
void engine_destroy(lt_engine *e);
lt_status engine_drop_cache(lt_engine *e);
// Resident mode: copy the graph to the device if it is not there yet.
lt_status engine_ensure_loaded(lt_engine *e);
lt_status engine_run(lt_engine *e, int app, int start, uint32_t source, uint64_t W, uint32_t length, uint32_t runs,
                     uint32_t run_base, float prob, uint64_t *counts_out, uint32_t *endpoints_out,
                     uint32_t *paths_out);
lt_status walk_device(int app, int start, const uint64_t *d_rowptr, const uint32_t *d_col, uint32_t V,
                      uint32_t source, uint64_t W, uint32_t length, float prob, uint32_t run, uint64_t seed,
                      uint64_t *d_counts, uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch,
                      uint64_t *d_stats, cudaStream_t st, int block_ctas);
size_t walk_scratch_bytes();
lt_status walk_device_compact(int app, int start, const uint32_t *d_rowptr32, const uint32_t *d_col, uint32_t V,
                              uint32_t source, uint64_t W, uint32_t length, float prob, uint32_t run, uint64_t seed,
                              uint32_t *d_counts32, uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch,
                              uint64_t *d_stats, cudaStream_t st, int ctas_per_sm);
lt_status rowptr_narrow(const uint64_t *d_rowptr, uint32_t *d_rowptr32, uint32_t V, cudaStream_t st);
lt_status walk_device_packed(int app, int start, uint32_t *d_rows, const uint32_t *d_col, uint32_t V, uint32_t source,
                             uint64_t W, uint32_t length, float prob, uint32_t run, uint64_t seed,
                             uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch, uint64_t *d_stats,
                             cudaStream_t st, int ctas_per_sm);
lt_status rows_pack(const uint64_t *d_rowptr, uint32_t *d_rows, uint32_t V, cudaStream_t st);
lt_status rows_counts(const uint32_t *d_rows, uint64_t *d_counts, uint32_t V, cudaStream_t st);
}  // namespace lt
