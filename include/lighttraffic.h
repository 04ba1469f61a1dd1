/*
 * lighttraffic.h -- C ABI of the GB300 random-walk engine.
 *
 * The reference (LightTraffic) has no FFI: its boundary is a compile-time
 * template plugin (struct Walker / App / AppManager, app/ppr.cu:11-94) driven
 * by LightTraffic<AppManager,App,Walker>::start (src/LightTraffic.h:11-44) and
 * configured from the command line by Config (src/Config.h:38-89).  Each entry
 * point below names the reference interface it replaces.
 *
 * Conventions
 *  - Every function returns lt_status; nothing calls exit() (the reference's
 *    gpuCall does, src/utils/GPUCall.h:3-11).  lt_last_error() gives a message
 *    for the most recent failure on the calling thread.
 *  - Output buffers are owned by the caller.  "host" buffers are ordinary or
 *    pinned host memory; "device" buffers are device pointers on the engine's
 *    GPU.
 *  - One engine per host thread; an engine is not re-entrant (the reference
 *    keeps static state in its scheduler too, src/Scheduler.h:394).
 *  - Types follow src/Type.h:5-8: vertex ids u32, edge offsets u64.  Visit
 *    counts are u64 (the reference's u32 counters overflow on hubs,
 *    app/pagerank.cu:133-135).
 *  - Randomness is Philox4x32-10 keyed by (seed, run, walker index, step
 *    value), never by thread or schedule, so results are bit-identical for
 *    every device cache size, scheduler and launch shape.
 */
#ifndef LIGHTTRAFFIC_H
#define LIGHTTRAFFIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lt_status {
    LT_OK = 0,
    LT_ERR_INVALID = 1,     /* bad argument */
    LT_ERR_IO = 2,          /* file cannot be opened / read / written */
    LT_ERR_FORMAT = 3,      /* truncated or inconsistent bcsr / .part file */
    LT_ERR_NOMEM = 4,       /* host or device allocation failed */
    LT_ERR_CUDA = 5,        /* a CUDA call failed */
    LT_ERR_PARTITION = 6,   /* one vertex does not fit the partition size */
    LT_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up */
    LT_ERR_CAPACITY = 8,    /* a device queue or buffer limit was exceeded */
    LT_ERR_UNSUPPORTED = 9, /* configuration this library does not support */
    LT_INTERRUPTED = 10     /* the run stopped at a checkpoint, as lt_engine_checkpoint asked */
} lt_status;

typedef enum lt_app { LT_APP_PPR = 0, LT_APP_PAGERANK = 1, LT_APP_WALK = 2 } lt_app;

/* Where walkers start.  SOURCE: all at one vertex (src/walk/SingleSource.h:6-20);
 * UNIFORM: a seeded uniform vertex each (src/walk/NodeSampler.h:5-15);
 * PER_VERTEX: walker i starts at vertex i mod V. */
typedef enum lt_start { LT_START_SOURCE = 0, LT_START_UNIFORM = 1, LT_START_PER_VERTEX = 2 } lt_start;

/* PLAIN: the reference policy, one partition per iteration
 * (src/Scheduler.h:84-171, :243-252, :368-388); FIFO: its FIFO_SCHE variant
 * (:113-127, :391-418).  The others run in waves: every step kernel drains
 * every cached partition's queue while the next loads stream in.  LEARNED:
 * cache slots go to the partitions the online-trained prefetcher network
 * predicts the most visits for; FREQUENCY: the same, scored by a moving
 * average of visits (ablation of the network); BATCHED: least recently used
 * slots (ablation of the predictions).  All give identical results. */
typedef enum lt_sched {
    LT_SCHED_PLAIN = 0,
    LT_SCHED_FIFO = 1,
    LT_SCHED_LEARNED = 2,
    LT_SCHED_FREQUENCY = 3,
    LT_SCHED_BATCHED = 4
} lt_sched;

typedef struct lt_graph lt_graph;
typedef struct lt_engine lt_engine;

typedef struct lt_graph_info {
    uint32_t num_nodes;          /* V */
    uint64_t num_edges;          /* E */
    uint32_t num_partitions;     /* P */
    uint64_t partition_bytes;    /* -s in bytes */
    uint32_t max_nodes_in_partition;
    uint64_t max_edges_in_partition;
} lt_graph_info;

typedef struct lt_engine_cfg {
    int device;                      /* CUDA device ordinal (the reference fixes 0, app/ppr.cu:101) */
    uint32_t num_device_partitions;  /* -p: the graph gets num_device_partitions x partition size bytes
                                        of device memory, as in the reference (src/GraphLoader.h:
                                        175-178); with resident_index the vertex index is paid from
                                        that budget, leaving fewer partition slots (0 = all cached) */
    uint64_t num_device_walkers;     /* -b: walkers held on the device (0 = all) */
    int sched;                       /* lt_sched */
    int pipeline;                    /* overlap partition loads with stepping (1 = on; 0 = loads
                                        finish first, the reference's NO_PIPELINE build,
                                        benchmark/figure13/Makefile): plain / FIFO compute other
                                        cached partitions while a load is in flight
                                        (src/Scheduler.h:194-208); wave runs overlap the next
                                        loads with the current step kernel */
    uint64_t zerocopy_threshold;     /* walkers below which a cold partition is read zero-copy;
                                        UINT64_MAX = default partitionSize/128/2 (src/Scheduler.h:295) */
    uint64_t seed;                   /* Philox key */
    int block_size;                  /* threads per CTA of the step kernel (0 = tuned default) */
    int ctas_per_sm;                 /* resident CTAs per SM (0 = occupancy maximum) */
    int resident_index;              /* out-of-core: keep the vertex index on the device (4 (V+1)
                                        bytes: each vertex's first edge as a u32 offset from its
                                        partition's first edge), so partition loads copy only edges and zero-copy
                                        hops read only col over the host link (1 = on, the default,
                                        falling back to 0 when the index does not fit in the -p
                                        budget with at least one slot beside it; 0 = the
                                        reference's layout, rowptr slices in the slots,
                                        src/GraphLoader.h:193-214) */
    uint64_t zc_group_bytes;         /* wave runs: estimated host bytes the partitions of one zero-copy
                                        group may touch (0 = 512 MiB; 128 MiB while serving) */
    uint64_t sweep_walkers;          /* wave runs: walkers left outside the cache at or below which one
                                        kernel reads every uncached partition zero-copy (0 = 2^14; 2^18 while serving) */
    uint32_t load_factor;            /* wave runs: a partition is loaded once its waiting walkers reach
                                        load_factor x zerocopy_threshold (0 = 256 / host bytes per
                                        zero-copy hop: 8 with the device index, 4 without) */
    int bucket_items;                /* bucketing tile: 16 (0) = 4096 walkers, 8 = 2048 */
    int no_prefill;                  /* wave runs: 1 = leave a cold cache to fill as walkers arrive
                                        instead of loading the policy's forecast set at a run's start */
    int hot_tier;                    /* wave runs with the device index: percent (0 = off, at most 90) of
                                        the graph budget left by the index that holds a hot-vertex tier,
                                        the adjacency of the vertices read most per byte outside the
                                        cache, chosen from the counts of the engine's first run of a
                                        walk and used by every later run (fewer partition slots) */
    int no_split;                    /* wave runs: 1 = one step kernel per pass; 0 (default) = while a
                                        zero-copy group is read, the walkers of cached queues and the ones
                                        created in the pass run in a concurrent kernel on one CTA per SM */
    int host_plan;                   /* out-of-core: 1 = the host plans every bucketing pass after
                                        reading the step kernel's histogram; 0 (default) = a device
                                        kernel plans it right behind the step kernel whenever the free
                                        chunks provably hold every arrival (same queues either way) */
} lt_engine_cfg;

typedef struct lt_stats {
    uint64_t updates;        /* App::update calls */
    uint64_t moves;          /* hops along an edge */
    uint64_t teleports;      /* PageRank jumps */
    uint64_t iterations;     /* scheduler iterations (src/Scheduler.h:314) */
    uint64_t explicit_iterations;
    uint64_t h2d_graph_bytes;
    uint64_t h2d_walker_bytes;
    uint64_t d2h_walker_bytes;
    uint64_t zerocopy_bytes;  /* host bytes read zero-copy per zero-copy hop, measured with ncu:
                                 32 B with the vertex index resident, 62 B without */
    uint64_t partition_loads;
    uint64_t kernel_launches;
    double running_ms;        /* host wall time of the run ("Running Time") */
    double graph_loading_ms;  /* event timers of src/Scheduler.h:284-288 */
    double computing_ms;
    double zerocopy_ms;
    double walker_loading_ms;
    double walker_evicting_ms;
    uint64_t graph_loading_calls;
    uint64_t computing_calls;
    uint64_t zerocopy_calls;
    uint64_t walker_loading_calls;
    uint64_t walker_evicting_calls;
    double step_kernel_ms;    /* CUDA-event time of the step kernels of the last run */
    uint64_t handoffs;        /* walkers staged and bucketed into another partition's queue */
    uint64_t overlap_computes; /* plain / FIFO loop: cached partitions computed while a load was in
                                  flight (getComputedPartition, src/Scheduler.h:194-208) */
    uint64_t zerocopy_groups;  /* wave runs: step kernels that read a bounded group of uncached
                                  partitions zero-copy */
    uint64_t zerocopy_sweeps;  /* wave runs: step kernels that read every uncached partition
                                  zero-copy to finish the last walkers */
    uint64_t cache_slots;      /* out of core: partition slots on the device */
    uint64_t index_on_device;  /* out of core: 1 when the vertex index is resident on the device */
    uint64_t refill_loads;     /* wave runs: loads that swapped a cached partition for one the
                                  policy forecasts more entries for */
    uint64_t prefill_loads;    /* wave runs: loads into a cold cache at a run's start, in the order of
                                  the policy's forecast (entries of its previous runs) */
    double bucket_ms;          /* CUDA-event time of the bucketing (scatter) kernels */
    double host_wait_ms;       /* host time blocked waiting for each iteration's step kernel */
    uint64_t device_plans;     /* bucketing passes planned on the device (the others by the host) */
    /* host time of the out-of-core loop outside waits, by phase (wave runs): */
    double host_sched_ms;      /* scheduling decisions before each step kernel */
    double host_submit_ms;     /* work list, plan inputs and launches of each pass */
    double host_replay_ms;     /* queue bookkeeping after each histogram read-back */
    double host_observe_ms;    /* kernel timers and the policy's per-iteration update */
    uint64_t split_launches;   /* passes whose step ran as two concurrent kernels */
    uint64_t hot_vertices;     /* vertices in the hot-vertex tier this run used (0: none) */
    double tier_build_ms;      /* host time building the tier after this run (0: not built) */
} lt_stats;

const char *lt_strerror(lt_status s);
const char *lt_last_error(void);
/* Library version string. */
const char *lt_version(void);

/* ------------------------------------------------------------------ graphs */

/* Open a .bcsr graph (src/GraphLoader.h:30-48) and its partition table.
 * materialize != 0: partition greedily with part_mb MiB partitions and write
 * <path>.part (Config -m, src/Config.h:63-66 + EqualSizeStrategy,
 * src/partition/PartitionStrategy.h:189-253,325-337); otherwise read
 * <path>.part (MaterializedStrategy, :76-97).  The graph is held in pinned
 * host memory (CPUGraph + cudaHostRegister, src/GraphLoader.h:115-157). */
lt_status lt_graph_open(const char *bcsr_path, int materialize, uint64_t part_mb, lt_graph **out);

/* Build a graph from caller CSR arrays (copied) and partition it with
 * part_bytes-byte partitions (EqualSizeStrategy(CPUBuffer&, maxSize),
 * src/partition/PartitionStrategy.h:239-241). */
lt_status lt_graph_from_csr(uint32_t num_nodes, uint64_t num_edges, const uint64_t *rowptr,
                            const uint32_t *col, uint64_t part_bytes, lt_graph **out);

/* Generate a seeded RMAT graph on the GPU (no counterpart in the reference,
 * whose datasets come from tools/convert_from_txt.cc): 2^scale raw vertices,
 * num_edges directed edges, quadrant probabilities a,b,c,d quantised to 2^-16;
 * isolated vertices removed keeping order (tools/rm_isolated_vertices.cc:70-87).
 * Self-loops and duplicate edges are kept. */
lt_status lt_graph_generate_rmat(int device, uint32_t scale, uint64_t num_edges, double a, double b,
                                 double c, double d, uint64_t seed, uint64_t part_bytes,
                                 lt_graph **out);

/* Build a graph from a text edge list (the reference's converter_txt,
 * tools/convert_from_txt.cc:66-218) and partition it with part_bytes-byte
 * partitions.  By default as the reference: lines not starting with a digit
 * are skipped, each line gives "source destination" (unsigned ids), self
 * loops are dropped, ids that appear in no edge are removed and the rest
 * renumbered in order, every edge is added in both directions, and the list
 * is sorted by (source, destination) with duplicates removed.  The flags
 * below switch steps off.  Write the result with lt_graph_write_bcsr. */
#define LT_EDGES_DIRECTED 1        /* keep edges one-way (no reverse edges) */
#define LT_EDGES_KEEP_DUPLICATES 2 /* keep repeated (source, destination) pairs */
#define LT_EDGES_KEEP_SELF_LOOPS 4
#define LT_EDGES_KEEP_ISOLATED 8   /* keep ids as given (below 2^32 - 1); V = largest id + 1 */
lt_status lt_graph_from_edge_list(const char *path, int flags, uint64_t part_bytes, lt_graph **out);

lt_status lt_graph_info_get(const lt_graph *g, lt_graph_info *out);
/* Copy the partition table: node_off[P+1], edge_off[P+1] (either may be NULL). */
lt_status lt_graph_partitions(const lt_graph *g, uint32_t *node_off, uint64_t *edge_off);
/* Host views of the CSR arrays (owned by the graph). */
lt_status lt_graph_csr(const lt_graph *g, const uint64_t **rowptr, const uint32_t **col);
lt_status lt_graph_write_bcsr(const lt_graph *g, const char *path);
/* Write <bcsr_path>.part for the graph's partition table (materialize, :325-337). */
lt_status lt_graph_write_part(const lt_graph *g, const char *bcsr_path);
void lt_graph_close(lt_graph *g);

/* Greedy partitioner on caller arrays (EqualSizeStrategy::init,
 * src/partition/PartitionStrategy.h:193-218).  node_off/edge_off hold cap
 * entries; on success *num_parts = P and entries [0, P] are written. */
lt_status lt_partition_equal_size(const uint64_t *rowptr, uint32_t num_nodes, uint64_t max_bytes,
                                  uint32_t *node_off, uint64_t *edge_off, uint32_t cap,
                                  uint32_t *num_parts);

/* ----------------------------------------------------------------- engines */

void lt_engine_cfg_default(lt_engine_cfg *cfg);
/* Replaces LightTraffic(Config&, AppManager&) + GPU/CPU device setup
 * (src/LightTraffic.h:19-31, src/Device.h:13-43). */
lt_status lt_engine_create(lt_graph *g, const lt_engine_cfg *cfg, lt_engine **out);
void lt_engine_destroy(lt_engine *e);
/* Drop every cached partition so the next run reloads them from the host. */
lt_status lt_engine_drop_cache(lt_engine *e);

/* PPR from one source (app/ppr.cu main + AppManager, :45-113): num_walkers
 * walks with stop probability prob; counts_out (host, u64[V], may be NULL)
 * receives per-vertex endpoint counts (AppManager::reduce, :65-67). */
lt_status lt_run_ppr(lt_engine *e, uint32_t source, uint64_t num_walkers, float prob,
                     uint64_t *counts_out);

/* Walk-based PageRank (app/pagerank.cu:160-219): runs epochs of num_walkers
 * walks of `length` updates each, teleport when U > alpha (alpha = 0.85 in the
 * reference, app/pagerank.cu:6); counts_out (host, u64[V], may be NULL). */
lt_status lt_run_pagerank(lt_engine *e, uint64_t num_walkers, uint32_t length, uint32_t runs,
                          float alpha, int start_mode, uint64_t *counts_out);

/* Fixed-length generic walk (app/genericwalk.cu:286-335) for run index `run`:
 * endpoints_out (host, u32[W]) and paths_out (host, u32[W*(length+1)],
 * INVALID 0xFFFFFFFF after a stop at a vertex without out-edges); either may
 * be NULL. */
lt_status lt_run_walk(lt_engine *e, uint64_t num_walkers, uint32_t length, uint32_t run,
                      int start_mode, uint32_t *endpoints_out, uint32_t *paths_out);

/* Statistics and phase timers of the last run (Scheduler::timing,
 * src/Scheduler.h:440-453). */
lt_status lt_engine_stats(const lt_engine *e, lt_stats *out);

/* ------------------------------------------------- checkpoint / resume */

/* Checkpoints of out-of-core runs (no counterpart in the reference, whose
 * runs cannot be resumed).  Once armed, every lt_run_* call on this engine
 * writes the run's state to `path` every `every` scheduler iterations
 * (replacing the previous file atomically); with stop != 0 the call returns
 * LT_INTERRUPTED right after the first checkpoint, as a preempted job would.
 * path = NULL disarms.  LT_ERR_UNSUPPORTED on an engine that holds the whole
 * graph (its runs are one kernel). */
lt_status lt_engine_checkpoint(lt_engine *e, const char *path, uint64_t every, int stop);

typedef struct lt_checkpoint_info {
    int app;                 /* lt_app */
    int start_mode;          /* lt_start */
    uint32_t source, length, runs, run_index;
    uint64_t num_walkers;
    uint32_t num_nodes;
    int has_endpoints, has_paths;
    uint64_t iteration;      /* scheduler iterations done when it was written */
} lt_checkpoint_info;

/* What a checkpoint file holds, for sizing the outputs of lt_resume. */
lt_status lt_checkpoint_read_info(const char *path, lt_checkpoint_info *out);

/* Finish the run saved in `path` on an out-of-core engine over the same
 * graph (any cache size, walker pool or scheduler) and write the outputs the
 * interrupted call would have written: counts u64[V] (PPR / PageRank),
 * endpoints u32[W] and paths u32[W*(length+1)] (generic walk, when the
 * original call asked for them).  The walks keep the checkpoint's seed, and
 * the results are those of a run that was never interrupted. */
lt_status lt_resume(lt_engine *e, const char *path, uint64_t *counts_out, uint32_t *endpoints_out,
                    uint32_t *paths_out);

/* ------------------------------------------------- device-resident kernels */

/* One pass of an app over a graph already resident in device memory, all
 * pointers on the current device, launched on `stream` (cudaStream_t, NULL =
 * legacy default stream).  This is the step kernel of randomWalkKernel
 * (src/WalkManager.h:229-246) over the whole graph at once.
 *   d_counts   : u64[V], added to (PPR / PageRank), may be NULL for LT_APP_WALK
 *   d_endpoints: u32[W] or NULL; d_paths: u32[W*(length+1)] or NULL (walk only)
 *   d_scratch  : device scratch of lt_walk_scratch_bytes() bytes; the call
 *                clears it on `stream` before the kernel.
 *   d_stats    : u64[3] or NULL: {updates, moves, teleports}, added to
 * prob is the PPR stop probability or the PageRank alpha.  Returns without
 * waiting for the kernel. */
size_t lt_walk_scratch_bytes(void);
lt_status lt_walk_device(int app, int start_mode, const uint64_t *d_rowptr, const uint32_t *d_col,
                         uint32_t num_nodes, uint32_t source, uint64_t num_walkers,
                         uint32_t length, float prob, uint32_t run, uint64_t seed,
                         uint64_t *d_counts, uint32_t *d_endpoints, uint32_t *d_paths,
                         void *d_scratch, uint64_t *d_stats, void *stream);

/* lt_walk_device on the compact layout: u32 row offsets (any graph with
 * E < 2^32; lt_rowptr_narrow makes them from the u64 ones) and u32 counters.
 * Same step kernel (src/WalkManager.h:229-246) and identical results; the two
 * arrays every update reuses take half the bytes, so they stay in L2.
 *   d_counts32 : u32[V], added to (PPR / PageRank); a call is rejected with
 *                LT_ERR_INVALID when its counter updates (W for PPR,
 *                W * length for PageRank) reach 2^32.  Counters that start at
 *                zero therefore cannot wrap within one call.
 * Other arguments as lt_walk_device. */
lt_status lt_walk_device_compact(int app, int start_mode, const uint32_t *d_rowptr32, const uint32_t *d_col,
                                 uint32_t num_nodes, uint32_t source, uint64_t num_walkers,
                                 uint32_t length, float prob, uint32_t run, uint64_t seed,
                                 uint32_t *d_counts32, uint32_t *d_endpoints, uint32_t *d_paths,
                                 void *d_scratch, uint64_t *d_stats, void *stream);
/* d_rowptr32[i] = d_rowptr[i] for i <= num_nodes (edge offsets below 2^32),
 * on `stream`. */
lt_status lt_rowptr_narrow(const uint64_t *d_rowptr, uint32_t *d_rowptr32, uint32_t num_nodes, void *stream);

/* lt_walk_device on the packed layout: d_rows = u32[2 (num_nodes + 1)],
 * d_rows[2v] the first edge of v (edge offsets below 2^32) and d_rows[2v+1]
 * v's counter (u32, added to; the same u32 overflow rule as
 * lt_walk_device_compact).  The row offsets an update reads and the counter
 * it increments share one 32-byte sector, so an update touches one sector
 * of vertex data instead of two.  Build d_rows with lt_rows_pack (counters
 * zeroed), read the counters with lt_rows_counts.  Same semantics as
 * randomWalkKernel (src/WalkManager.h:229-246); the layout has no
 * counterpart in the reference. */
lt_status lt_walk_device_packed(int app, int start_mode, uint32_t *d_rows, const uint32_t *d_col, uint32_t num_nodes,
                                uint32_t source, uint64_t num_walkers, uint32_t length, float prob, uint32_t run,
                                uint64_t seed, uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch,
                                uint64_t *d_stats, void *stream);
/* d_rows[2i] = d_rowptr[i] (i <= num_nodes), d_rows[2i+1] = 0, on `stream`. */
lt_status lt_rows_pack(const uint64_t *d_rowptr, uint32_t *d_rows, uint32_t num_nodes, void *stream);
/* d_counts[v] = d_rows[2v+1] (v < num_nodes), widened to u64, on `stream`. */
lt_status lt_rows_counts(const uint32_t *d_rows, uint64_t *d_counts, uint32_t num_nodes, void *stream);

/* lt_walk_device without the scratch argument, for callers that cannot
 * allocate device memory: a plugin whose host framework owns every device
 * allocation and hands over only inputs and outputs, or a process whose
 * device memory another allocator has reserved in full.  No counterpart in
 * the reference.  It allocates nothing: its scratch is a 256-byte static
 * device array shared by every call in the process; the call clears it on
 * `stream` first, calls that overlap on the GPU race (order them on one
 * stream), and a scratch need above 256 bytes is rejected with
 * LT_ERR_CAPACITY.  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress) and keeps it for the life of the process;
 * make that first call before any stream capture begins, and do not call
 * cudaDeviceReset on a device this entry point has used (the kept address
 * would then be stale). */
lt_status lt_walk_device_noalloc(int app, int start_mode, const uint64_t *d_rowptr, const uint32_t *d_col,
                                 uint32_t num_nodes, uint32_t source, uint64_t num_walkers,
                                 uint32_t length, float prob, uint32_t run, uint64_t seed,
                                 uint64_t *d_counts, uint32_t *d_endpoints, uint32_t *d_paths,
                                 uint64_t *d_stats, void *stream);

/* ------------------------------------------------- batched multi-source PPR */

/* Many PPR queries in one persistent launch (no counterpart in the
 * reference, which runs one source per process, app/ppr.cu:96-113).  Query q
 * runs walkers[q] walks from sources[q] keyed by seeds[q] (NULL: the engine
 * seed for every query), so its counts equal lt_run_ppr(sources[q],
 * walkers[q]) on an engine with that seed, alone or in any batch.  Output:
 * the (vertex, count) pairs of query q are out_vertices / out_counts
 * [out_offsets[q], out_offsets[q+1]), u32 counts, pairs of one query in
 * unspecified order.  out_offsets holds n+1 entries; out_capacity must be at
 * least the sum of walkers[].  Needs every partition cached on the device.
 * The batch pipeline is captured in a CUDA graph on first use and replayed. */
lt_status lt_ppr_batch(lt_engine *e, uint32_t n, const uint32_t *sources, const uint64_t *walkers,
                       const uint64_t *seeds, float prob, uint64_t *out_offsets, uint32_t *out_vertices,
                       uint32_t *out_counts, uint64_t out_capacity);
/* The same on device buffers, on `stream`; returns without waiting. */
lt_status lt_ppr_batch_device(lt_engine *e, uint32_t n, const uint32_t *d_sources, const uint64_t *d_walkers,
                              const uint64_t *d_seeds, float prob, uint64_t *d_out_offsets,
                              uint32_t *d_out_vertices, uint32_t *d_out_counts, uint64_t out_capacity,
                              void *stream);

typedef struct lt_batch_tune {
    int block;        /* threads per CTA of the walk kernel */
    int ctas_per_sm;  /* 0 = occupancy maximum */
    int load_shift;   /* per-query table capacity = next_pow2(walkers << load_shift) */
    int tuned;        /* 1 once lt_engine_autotune ran */
} lt_batch_tune;

/* Resident engine: time the batch pipeline on a synthetic batch for each
 * block size and table load factor and keep the fastest.  Out-of-core
 * engine: time cold-cache PPR trial runs and tune, one knob at a time, the
 * zero-copy group footprint, the load threshold factor, the step kernel's
 * CTAs per SM and the bucketing tile (lt_engine_ooc_tune reports them).
 * Results never depend on these choices. */
lt_status lt_engine_autotune(lt_engine *e);

typedef struct lt_ooc_tune {
    int tuned;                /* 1 once lt_engine_autotune ran on an out-of-core engine */
    uint64_t trial_walkers;   /* walkers of each trial run */
    uint64_t zc_group_bytes;  /* chosen lt_engine_cfg values (0 = default) */
    uint32_t load_factor;
    int ctas_per_sm;
    int bucket_items;
    double default_ms;        /* trial run time with the values before tuning */
    double tuned_ms;          /* with the chosen values */
} lt_ooc_tune;
lt_status lt_engine_ooc_tune(const lt_engine *e, lt_ooc_tune *out);
lt_status lt_engine_batch_tune(const lt_engine *e, lt_batch_tune *out);

/* ------------------------------------------------------------------ serving */

/* Continuous-batching PPR server on an out-of-core engine (no counterpart in
 * the reference, which runs one source per process).  Queries are admitted
 * when a query slot, room in the table arena (table_slots entries of 8 bytes)
 * and walker-pool chunks for all their walkers are free; admitted queries
 * share every scheduler iteration, cached partition and kernel launch with
 * the queries already running; their walkers stay in the device pool.  Each
 * query's counts depend only on (source, walkers, seed, prob). */
typedef struct lt_server lt_server;
lt_status lt_serve_open(lt_engine *e, uint32_t max_active, uint64_t table_slots, float prob, lt_server **out);
/* Queue a query; arrival_ms (lt_serve_now_ms clock, <= 0: now) starts its latency clock. */
lt_status lt_serve_submit(lt_server *s, uint32_t source, uint64_t walkers, uint64_t seed, double arrival_ms,
                          uint64_t *ticket);
/* Admit what fits, run one scheduler iteration, extract finished queries. */
lt_status lt_serve_step(lt_server *s, uint32_t *completed, uint32_t *active, uint32_t *pending);
/* done = 1 once the query finished; with vertices / counts given (capacity
 * pairs), copy its (vertex, count) pairs (unspecified order) and release it. */
lt_status lt_serve_result(lt_server *s, uint64_t ticket, int *done, uint64_t *n_pairs, uint32_t *vertices,
                          uint32_t *counts, uint64_t capacity, double *latency_ms);
/* Tickets of queries finished since the last call (up to cap); returns how many were written. */
uint64_t lt_serve_finished(lt_server *s, uint64_t *tickets, uint64_t cap);
void lt_serve_close(lt_server *s);
double lt_serve_now_ms(void);

/* ------------------------------------------------------ learned prefetcher */

typedef struct lt_policy_stats {
    char name[16];          /* "plain", "fifo", "learned", "frequency" */
    uint64_t train_steps;   /* SGD steps taken by the prefetcher network */
    double net_loss;        /* mean squared error of the network on the last half of its training batches */
    double baseline_loss;   /* the same for the moving-average predictor on those batches */
    uint64_t predictions;   /* prediction passes consumed by the policy */
    uint64_t net_used;      /* of those, passes that used the network's forecast (its running validation
                               loss below the moving average's); the others used the moving average */
} lt_policy_stats;

/* Scheduling-policy statistics of the engine's last out-of-core runs.  No
 * counterpart in the reference. */
lt_status lt_engine_policy_stats(const lt_engine *e, lt_policy_stats *out);

/* ------------------------------------------------------------ ABI layout */

/* Offset and size of a field of one of this header's structs, by name
 * ("lt_engine_cfg", "num_device_walkers"), and the size of a struct, for
 * bindings that mirror the structs (a cgo, JNI or ctypes layer can check its
 * copy against the library it loads).  LT_ERR_INVALID / 0 for unknown
 * names.  No GPU needed. */
lt_status lt_abi_field(const char *type, const char *field, size_t *offset, size_t *size);
size_t lt_abi_sizeof(const char *type);

/* Per partition, over the engine's last out-of-core run: walkers that
 * entered it, those that entered while it was cached, and step-kernel
 * launches during which it was cached (P entries each; any may be NULL).
 * What a cache policy could gain is read off these.  No counterpart in the
 * reference. */
lt_status lt_engine_partition_stats(const lt_engine *e, uint64_t *visits, uint64_t *cached_visits,
                                    uint64_t *cached_launches);

/* Forward and backward pass (and, when lr > 0, one SGD-with-momentum step) of
 * the learned prefetcher's network on caller data, on `device`: a 2-layer FP32
 * MLP with 16 inputs, 64 ReLU units and one output, mean squared error loss.
 * params / grad_out / params_out use the layout W1[i*64+j] | b1[64] | W2[64] |
 * b2 (1153 floats); x is n*16, y / pred_out are n.  No counterpart in the
 * reference (its scheduler has no learned component); exposed so the kernels
 * can be checked against a CPU implementation. */
lt_status lt_mlp_check(int device, uint32_t n, const float *x, const float *y, const float *params, float lr,
                       float momentum, float *pred_out, float *grad_out, float *loss_out, float *params_out);

/* Pinned host -> device copy bandwidth of `device` in GB/s (best of five
 * 1 GiB copies): the host-link roofline of out-of-core runs.  No counterpart
 * in the reference. */
lt_status lt_host_link_gbs(int device, double *gbs);

/* Page-locked host memory (portable, mapped) for the host buffers of the
 * lt_run_* / lt_ppr_batch calls: results then come back at the link's speed
 * instead of through the driver's staging copies into pageable memory.  No
 * counterpart in the reference. */
lt_status lt_host_alloc(uint64_t bytes, void **out);
/* Random-read rate of the GPU from a mapped pinned host buffer of `bytes`
 * (0 = 2 GiB), in GB/s of the 32-byte sectors the link moves (one per
 * zero-copy hop): the ceiling of the zero-copy step kernels.  No counterpart
 * in the reference. */
lt_status lt_host_gather_gbs(int device, uint64_t bytes, double *gbs);
void lt_host_free(void *p);

/* The remainder x[i] % d[i] as the walk kernels compute it (host build of the
 * same code), for checking it against native division.  No counterpart in
 * the reference. */
lt_status lt_mod_check(uint64_t n, const uint64_t *x, const uint64_t *d, uint64_t *out);
/* The same remainder computed by the device build (device buffers, on
 * `stream`; a zero divisor gives UINT64_MAX).  No counterpart in the
 * reference. */
lt_status lt_mod_check_device(uint64_t n, const uint64_t *d_x, const uint64_t *d_d, uint64_t *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* LIGHTTRAFFIC_H */
