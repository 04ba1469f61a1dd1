// capi.cpp -- extern "C" entry points declared in include/lighttraffic.h.
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <new>

#include "engine.h"
#include "lt_core.cuh"

using namespace lt;

// ---- layout of the ABI structs, for bindings that mirror them (the Python
// package checks its ctypes mirror against this table)

namespace {
struct AbiField {
    const char *type, *field;
    size_t offset, size;
};
#define LT_ABI_FIELD(T, F) {#T, #F, offsetof(T, F), sizeof(((T *)nullptr)->F)}
const AbiField kAbiFields[] = {
    LT_ABI_FIELD(lt_graph_info, num_nodes),
    LT_ABI_FIELD(lt_graph_info, num_edges),
    LT_ABI_FIELD(lt_graph_info, num_partitions),
    LT_ABI_FIELD(lt_graph_info, partition_bytes),
    LT_ABI_FIELD(lt_graph_info, max_nodes_in_partition),
    LT_ABI_FIELD(lt_graph_info, max_edges_in_partition),
    LT_ABI_FIELD(lt_engine_cfg, device),
    LT_ABI_FIELD(lt_engine_cfg, num_device_partitions),
    LT_ABI_FIELD(lt_engine_cfg, num_device_walkers),
    LT_ABI_FIELD(lt_engine_cfg, sched),
    LT_ABI_FIELD(lt_engine_cfg, pipeline),
    LT_ABI_FIELD(lt_engine_cfg, zerocopy_threshold),
    LT_ABI_FIELD(lt_engine_cfg, seed),
    LT_ABI_FIELD(lt_engine_cfg, block_size),
    LT_ABI_FIELD(lt_engine_cfg, ctas_per_sm),
    LT_ABI_FIELD(lt_engine_cfg, resident_index),
    LT_ABI_FIELD(lt_engine_cfg, zc_group_bytes),
    LT_ABI_FIELD(lt_engine_cfg, sweep_walkers),
    LT_ABI_FIELD(lt_engine_cfg, load_factor),
    LT_ABI_FIELD(lt_engine_cfg, bucket_items),
    LT_ABI_FIELD(lt_engine_cfg, no_prefill),
    LT_ABI_FIELD(lt_engine_cfg, hot_tier),
    LT_ABI_FIELD(lt_engine_cfg, no_split),
    LT_ABI_FIELD(lt_engine_cfg, host_plan),
    LT_ABI_FIELD(lt_stats, updates),
    LT_ABI_FIELD(lt_stats, moves),
    LT_ABI_FIELD(lt_stats, teleports),
    LT_ABI_FIELD(lt_stats, iterations),
    LT_ABI_FIELD(lt_stats, explicit_iterations),
    LT_ABI_FIELD(lt_stats, h2d_graph_bytes),
    LT_ABI_FIELD(lt_stats, h2d_walker_bytes),
    LT_ABI_FIELD(lt_stats, d2h_walker_bytes),
    LT_ABI_FIELD(lt_stats, zerocopy_bytes),
    LT_ABI_FIELD(lt_stats, partition_loads),
    LT_ABI_FIELD(lt_stats, kernel_launches),
    LT_ABI_FIELD(lt_stats, running_ms),
    LT_ABI_FIELD(lt_stats, graph_loading_ms),
    LT_ABI_FIELD(lt_stats, computing_ms),
    LT_ABI_FIELD(lt_stats, zerocopy_ms),
    LT_ABI_FIELD(lt_stats, walker_loading_ms),
    LT_ABI_FIELD(lt_stats, walker_evicting_ms),
    LT_ABI_FIELD(lt_stats, graph_loading_calls),
    LT_ABI_FIELD(lt_stats, computing_calls),
    LT_ABI_FIELD(lt_stats, zerocopy_calls),
    LT_ABI_FIELD(lt_stats, walker_loading_calls),
    LT_ABI_FIELD(lt_stats, walker_evicting_calls),
    LT_ABI_FIELD(lt_stats, step_kernel_ms),
    LT_ABI_FIELD(lt_stats, handoffs),
    LT_ABI_FIELD(lt_stats, overlap_computes),
    LT_ABI_FIELD(lt_stats, zerocopy_groups),
    LT_ABI_FIELD(lt_stats, zerocopy_sweeps),
    LT_ABI_FIELD(lt_stats, cache_slots),
    LT_ABI_FIELD(lt_stats, index_on_device),
    LT_ABI_FIELD(lt_stats, refill_loads),
    LT_ABI_FIELD(lt_stats, prefill_loads),
    LT_ABI_FIELD(lt_stats, bucket_ms),
    LT_ABI_FIELD(lt_stats, host_wait_ms),
    LT_ABI_FIELD(lt_stats, device_plans),
    LT_ABI_FIELD(lt_stats, host_sched_ms),
    LT_ABI_FIELD(lt_stats, host_submit_ms),
    LT_ABI_FIELD(lt_stats, host_replay_ms),
    LT_ABI_FIELD(lt_stats, host_observe_ms),
    LT_ABI_FIELD(lt_stats, split_launches),
    LT_ABI_FIELD(lt_stats, hot_vertices),
    LT_ABI_FIELD(lt_stats, tier_build_ms),
    LT_ABI_FIELD(lt_checkpoint_info, app),
    LT_ABI_FIELD(lt_checkpoint_info, start_mode),
    LT_ABI_FIELD(lt_checkpoint_info, source),
    LT_ABI_FIELD(lt_checkpoint_info, length),
    LT_ABI_FIELD(lt_checkpoint_info, runs),
    LT_ABI_FIELD(lt_checkpoint_info, run_index),
    LT_ABI_FIELD(lt_checkpoint_info, num_walkers),
    LT_ABI_FIELD(lt_checkpoint_info, num_nodes),
    LT_ABI_FIELD(lt_checkpoint_info, has_endpoints),
    LT_ABI_FIELD(lt_checkpoint_info, has_paths),
    LT_ABI_FIELD(lt_checkpoint_info, iteration),
    LT_ABI_FIELD(lt_batch_tune, block),
    LT_ABI_FIELD(lt_batch_tune, ctas_per_sm),
    LT_ABI_FIELD(lt_batch_tune, load_shift),
    LT_ABI_FIELD(lt_batch_tune, tuned),
    LT_ABI_FIELD(lt_ooc_tune, tuned),
    LT_ABI_FIELD(lt_ooc_tune, trial_walkers),
    LT_ABI_FIELD(lt_ooc_tune, zc_group_bytes),
    LT_ABI_FIELD(lt_ooc_tune, load_factor),
    LT_ABI_FIELD(lt_ooc_tune, ctas_per_sm),
    LT_ABI_FIELD(lt_ooc_tune, bucket_items),
    LT_ABI_FIELD(lt_ooc_tune, default_ms),
    LT_ABI_FIELD(lt_ooc_tune, tuned_ms),
    LT_ABI_FIELD(lt_policy_stats, name),
    LT_ABI_FIELD(lt_policy_stats, train_steps),
    LT_ABI_FIELD(lt_policy_stats, net_loss),
    LT_ABI_FIELD(lt_policy_stats, baseline_loss),
    LT_ABI_FIELD(lt_policy_stats, predictions),
    LT_ABI_FIELD(lt_policy_stats, net_used),
};
#undef LT_ABI_FIELD
const struct {
    const char *type;
    size_t size;
} kAbiTypes[] = {
    {"lt_graph_info", sizeof(lt_graph_info)},
    {"lt_engine_cfg", sizeof(lt_engine_cfg)},
    {"lt_stats", sizeof(lt_stats)},
    {"lt_checkpoint_info", sizeof(lt_checkpoint_info)},
    {"lt_batch_tune", sizeof(lt_batch_tune)},
    {"lt_ooc_tune", sizeof(lt_ooc_tune)},
    {"lt_policy_stats", sizeof(lt_policy_stats)},
};
}  // namespace


extern "C" {

const char *lt_strerror(lt_status s)
{
    switch (s) {
    case LT_OK: return "ok";
    case LT_ERR_INVALID: return "invalid argument";
    case LT_ERR_IO: return "i/o error";
    case LT_ERR_FORMAT: return "malformed file";
    case LT_ERR_NOMEM: return "out of memory";
    case LT_ERR_CUDA: return "CUDA error";
    case LT_ERR_PARTITION: return "vertex does not fit the partition size";
    case LT_ERR_TIMEOUT: return "bounded device wait expired";
    case LT_ERR_CAPACITY: return "capacity exceeded";
    case LT_ERR_UNSUPPORTED: return "unsupported configuration";
    case LT_INTERRUPTED: return "run stopped at a checkpoint";
    }
    return "unknown status";
}

const char *lt_last_error(void) { return last_error(); }
const char *lt_version(void) { return "lighttraffic-gb300 0.1 (sm_103a)"; }

lt_status lt_partition_equal_size(const uint64_t *rowptr, uint32_t num_nodes, uint64_t max_bytes, uint32_t *node_off,
                                  uint64_t *edge_off, uint32_t cap, uint32_t *num_parts)
{
    if (!rowptr || !node_off || !edge_off || !num_parts) return fail(LT_ERR_INVALID, "null argument");
    std::vector<uint32_t> no;
    std::vector<uint64_t> eo;
    LT_TRY(partition_equal_size(rowptr, num_nodes, max_bytes, no, eo));
    if (no.size() > cap) return fail(LT_ERR_CAPACITY, "%zu partitions exceed the output capacity %u", no.size() - 1, cap);
    std::memcpy(node_off, no.data(), 4 * no.size());
    std::memcpy(edge_off, eo.data(), 8 * eo.size());
    *num_parts = (uint32_t)no.size() - 1;
    return LT_OK;
}

lt_status lt_graph_open(const char *bcsr_path, int materialize, uint64_t part_mb, lt_graph **out)
{
    if (!bcsr_path || !out) return fail(LT_ERR_INVALID, "null argument");
    lt_graph *g = new (std::nothrow) lt_graph();
    if (!g) return fail(LT_ERR_NOMEM, "graph allocation failed");
    lt_status s = read_bcsr(bcsr_path, *g);
    if (s == LT_OK) {
        if (materialize) {
            g->part_bytes = part_mb * 1024ull * 1024ull;
            s = partition_equal_size(g->rowptr(), g->V, g->part_bytes, g->node_off, g->edge_off);
            if (s == LT_OK) s = finish_partitions(*g);
            if (s == LT_OK) s = write_part(*g, bcsr_path);
        } else {
            s = read_part(bcsr_path, *g);
            if (s == LT_OK && g->node_off.back() != g->V)
                s = fail(LT_ERR_FORMAT, "partition file does not match the graph");
        }
    }
    if (s != LT_OK) {
        graph_free(*g);
        delete g;
        return s;
    }
    *out = g;
    return LT_OK;
}

lt_status lt_graph_from_edge_list(const char *path, int flags, uint64_t part_bytes, lt_graph **out)
{
    if (!path || !out) return fail(LT_ERR_INVALID, "null argument");
    if (flags & ~(LT_EDGES_DIRECTED | LT_EDGES_KEEP_DUPLICATES | LT_EDGES_KEEP_SELF_LOOPS | LT_EDGES_KEEP_ISOLATED))
        return fail(LT_ERR_INVALID, "unknown edge-list flags %d", flags);
    lt_graph *g = new (std::nothrow) lt_graph();
    if (!g) return fail(LT_ERR_NOMEM, "graph allocation failed");
    lt_status s = read_edge_list(path, flags, *g);
    if (s == LT_OK) {
        g->part_bytes = part_bytes;
        s = partition_equal_size(g->rowptr(), g->V, part_bytes, g->node_off, g->edge_off);
    }
    if (s == LT_OK) s = finish_partitions(*g);
    if (s != LT_OK) {
        graph_free(*g);
        delete g;
        return s;
    }
    *out = g;
    return LT_OK;
}

lt_status lt_graph_from_csr(uint32_t num_nodes, uint64_t num_edges, const uint64_t *rowptr, const uint32_t *col,
                            uint64_t part_bytes, lt_graph **out)
{
    if (!rowptr || (!col && num_edges) || !out || num_nodes == 0) return fail(LT_ERR_INVALID, "null or empty argument");
    if (rowptr[0] != 0 || rowptr[num_nodes] != num_edges) return fail(LT_ERR_FORMAT, "rowptr does not span [0, E]");
    lt_graph *g = new (std::nothrow) lt_graph();
    if (!g) return fail(LT_ERR_NOMEM, "graph allocation failed");
    g->V = num_nodes;
    g->E = num_edges;
    lt_status s = host_alloc(g->rowptr_buf, 8ull * ((uint64_t)num_nodes + 1), true);
    if (s == LT_OK) s = host_alloc(g->col_buf, 4ull * num_edges, true);
    if (s == LT_OK) {
        std::memcpy(g->rowptr_mut(), rowptr, 8ull * ((uint64_t)num_nodes + 1));
        if (num_edges) std::memcpy(g->col_mut(), col, 4ull * num_edges);
        for (uint64_t v = 0; v < num_nodes && s == LT_OK; v++)
            if (rowptr[v + 1] < rowptr[v]) s = fail(LT_ERR_FORMAT, "rowptr decreases at %llu", (unsigned long long)v);
        for (uint64_t k = 0; k < num_edges && s == LT_OK; k++)
            if (col[k] >= num_nodes) s = fail(LT_ERR_FORMAT, "col[%llu] out of range", (unsigned long long)k);
    }
    if (s == LT_OK) {
        g->part_bytes = part_bytes;
        s = partition_equal_size(g->rowptr(), g->V, part_bytes, g->node_off, g->edge_off);
    }
    if (s == LT_OK) s = finish_partitions(*g);
    if (s != LT_OK) {
        graph_free(*g);
        delete g;
        return s;
    }
    *out = g;
    return LT_OK;
}

lt_status lt_graph_generate_rmat(int device, uint32_t scale, uint64_t num_edges, double a, double b, double c, double d,
                                 uint64_t seed, uint64_t part_bytes, lt_graph **out)
{
    if (!out) return fail(LT_ERR_INVALID, "null output");
    lt_graph *g = new (std::nothrow) lt_graph();
    if (!g) return fail(LT_ERR_NOMEM, "graph allocation failed");
    lt_status s = generate_rmat(device, scale, num_edges, a, b, c, d, seed, *g);
    if (s == LT_OK) {
        g->part_bytes = part_bytes;
        s = partition_equal_size(g->rowptr(), g->V, part_bytes, g->node_off, g->edge_off);
    }
    if (s == LT_OK) s = finish_partitions(*g);
    if (s != LT_OK) {
        graph_free(*g);
        delete g;
        return s;
    }
    *out = g;
    return LT_OK;
}

lt_status lt_graph_info_get(const lt_graph *g, lt_graph_info *out)
{
    if (!g || !out) return fail(LT_ERR_INVALID, "null argument");
    out->num_nodes = g->V;
    out->num_edges = g->E;
    out->num_partitions = g->P();
    out->partition_bytes = g->part_bytes;
    out->max_nodes_in_partition = g->max_nodes;
    out->max_edges_in_partition = g->max_edges;
    return LT_OK;
}

lt_status lt_graph_partitions(const lt_graph *g, uint32_t *node_off, uint64_t *edge_off)
{
    if (!g) return fail(LT_ERR_INVALID, "null graph");
    if (node_off) std::memcpy(node_off, g->node_off.data(), 4 * g->node_off.size());
    if (edge_off) std::memcpy(edge_off, g->edge_off.data(), 8 * g->edge_off.size());
    return LT_OK;
}

lt_status lt_graph_csr(const lt_graph *g, const uint64_t **rowptr, const uint32_t **col)
{
    if (!g) return fail(LT_ERR_INVALID, "null graph");
    if (rowptr) *rowptr = g->rowptr();
    if (col) *col = g->col();
    return LT_OK;
}

lt_status lt_graph_write_bcsr(const lt_graph *g, const char *path)
{
    if (!g || !path) return fail(LT_ERR_INVALID, "null argument");
    return write_bcsr(*g, path);
}

lt_status lt_graph_write_part(const lt_graph *g, const char *bcsr_path)
{
    if (!g || !bcsr_path) return fail(LT_ERR_INVALID, "null argument");
    return write_part(*g, bcsr_path);
}

void lt_graph_close(lt_graph *g)
{
    if (!g) return;
    graph_free(*g);
    delete g;
}

void lt_engine_cfg_default(lt_engine_cfg *cfg)
{
    if (!cfg) return;
    std::memset(cfg, 0, sizeof *cfg);
    cfg->device = 0;
    cfg->num_device_partitions = 0;
    cfg->num_device_walkers = 0;
    cfg->sched = LT_SCHED_PLAIN;
    cfg->pipeline = 1;
    cfg->zerocopy_threshold = UINT64_MAX;
    cfg->seed = 0x5EED5EEDull;
    cfg->block_size = 0;
    cfg->ctas_per_sm = 0;
    cfg->resident_index = 1;
}

lt_status lt_engine_create(lt_graph *g, const lt_engine_cfg *cfg, lt_engine **out)
{
    lt_engine_cfg c;
    lt_engine_cfg_default(&c);
    if (cfg) c = *cfg;
    return engine_create(g, c, out);
}

void lt_engine_destroy(lt_engine *e) { engine_destroy(e); }

lt_status lt_engine_drop_cache(lt_engine *e)
{
    if (!e) return fail(LT_ERR_INVALID, "null engine");
    return engine_drop_cache(e);
}

lt_status lt_run_ppr(lt_engine *e, uint32_t source, uint64_t num_walkers, float prob, uint64_t *counts_out)
{
    if (!e) return fail(LT_ERR_INVALID, "null engine");
    if (!(prob > 0.0f && prob <= 1.0f)) return fail(LT_ERR_INVALID, "PPR stop probability must be in (0, 1]");
    return engine_run(e, LT_APP_PPR, LT_START_SOURCE, source, num_walkers, 0, 1, 0, prob, counts_out, nullptr, nullptr);
}

lt_status lt_run_pagerank(lt_engine *e, uint64_t num_walkers, uint32_t length, uint32_t runs, float alpha,
                          int start_mode, uint64_t *counts_out)
{
    if (!e) return fail(LT_ERR_INVALID, "null engine");
    if (length == 0) return fail(LT_ERR_INVALID, "walk length must be positive");
    if (start_mode == LT_START_SOURCE) return fail(LT_ERR_INVALID, "PageRank walkers start uniformly or per vertex");
    return engine_run(e, LT_APP_PAGERANK, start_mode, 0, num_walkers, length, runs, 0, alpha, counts_out, nullptr, nullptr);
}

lt_status lt_run_walk(lt_engine *e, uint64_t num_walkers, uint32_t length, uint32_t run, int start_mode,
                      uint32_t *endpoints_out, uint32_t *paths_out)
{
    if (!e) return fail(LT_ERR_INVALID, "null engine");
    if (length == 0) return fail(LT_ERR_INVALID, "walk length must be positive");
    if (start_mode == LT_START_SOURCE) return fail(LT_ERR_INVALID, "generic walkers start uniformly or per vertex");
    return engine_run(e, LT_APP_WALK, start_mode, 0, num_walkers, length, 1, run, 0.0f, nullptr, endpoints_out, paths_out);
}

lt_status lt_engine_stats(const lt_engine *e, lt_stats *out)
{
    if (!e || !out) return fail(LT_ERR_INVALID, "null argument");
    *out = e->stats;
    return LT_OK;
}

lt_status lt_engine_policy_stats(const lt_engine *e, lt_policy_stats *out)
{
    if (!e || !out) return fail(LT_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof *out);
    if (!e->ooc) {
        std::strncpy(out->name, "resident", sizeof out->name - 1);
        return LT_OK;
    }
    ooc_policy_stats(e->ooc, *out);
    return LT_OK;
}

lt_status lt_engine_partition_stats(const lt_engine *e, uint64_t *visits, uint64_t *cached_visits,
                                    uint64_t *cached_launches)
{
    if (!e) return fail(LT_ERR_INVALID, "null argument");
    if (!e->ooc) return fail(LT_ERR_UNSUPPORTED, "partition statistics are kept by out-of-core engines");
    ooc_partition_stats(e->ooc, visits, cached_visits, cached_launches);
    return LT_OK;
}

size_t lt_walk_scratch_bytes(void) { return walk_scratch_bytes(); }

lt_status lt_host_link_gbs(int device, double *gbs)
{
    if (!gbs) return fail(LT_ERR_INVALID, "null argument");
    LT_CUDA_TRY(cudaSetDevice(device));
    const size_t n = size_t(1) << 30;
    void *h = nullptr, *d = nullptr;
    LT_CUDA_TRY(cudaHostAlloc(&h, n, cudaHostAllocDefault));
    if (cudaMalloc(&d, n) != cudaSuccess) {
        cudaFreeHost(h);
        return fail(LT_ERR_NOMEM, "cudaMalloc of 1 GiB failed");
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double best = 0;
    for (int i = 0; i < 5; i++) {
        cudaEventRecord(a, 0);
        cudaMemcpyAsync(d, h, n, cudaMemcpyHostToDevice, 0);
        cudaEventRecord(b, 0);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms > 0) best = std::max(best, (double)n / (ms / 1e3) / 1e9);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    cudaFreeHost(h);
    *gbs = best;
    return cudaGetLastError() == cudaSuccess ? LT_OK : fail(LT_ERR_CUDA, "bandwidth probe failed");
}

lt_status lt_mod_check(uint64_t n, const uint64_t *x, const uint64_t *d, uint64_t *out)
{
    if (!x || !d || !out) return fail(LT_ERR_INVALID, "null argument");
    for (uint64_t i = 0; i < n; i++) {
        if (d[i] == 0) return fail(LT_ERR_INVALID, "zero divisor at %llu", (unsigned long long)i);
        out[i] = mod_u64(x[i], d[i]);
    }
    return LT_OK;
}

lt_status lt_ppr_batch(lt_engine *e, uint32_t n, const uint32_t *sources, const uint64_t *walkers,
                       const uint64_t *seeds, float prob, uint64_t *out_offsets, uint32_t *out_vertices,
                       uint32_t *out_counts, uint64_t out_capacity)
{
    if (!e || !sources || !walkers || !out_offsets || !out_vertices || !out_counts)
        return fail(LT_ERR_INVALID, "null argument");
    return batch_run(e, n, sources, walkers, seeds, prob, out_offsets, out_vertices, out_counts, out_capacity);
}

lt_status lt_ppr_batch_device(lt_engine *e, uint32_t n, const uint32_t *d_sources, const uint64_t *d_walkers,
                              const uint64_t *d_seeds, float prob, uint64_t *d_out_offsets,
                              uint32_t *d_out_vertices, uint32_t *d_out_counts, uint64_t out_capacity,
                              void *stream)
{
    if (!e || !d_sources || !d_walkers || !d_seeds || !d_out_offsets || !d_out_vertices || !d_out_counts)
        return fail(LT_ERR_INVALID, "null argument");
    return batch_run_device(e, n, d_sources, d_walkers, d_seeds, prob, d_out_offsets, d_out_vertices, d_out_counts,
                            out_capacity, (cudaStream_t)stream);
}

lt_status lt_serve_open(lt_engine *e, uint32_t max_active, uint64_t table_slots, float prob, lt_server **out)
{
    if (!e || !out) return fail(LT_ERR_INVALID, "null argument");
    return serve_open(e, max_active, table_slots, prob, out);
}

lt_status lt_serve_submit(lt_server *s, uint32_t source, uint64_t walkers, uint64_t seed, double arrival_ms,
                          uint64_t *ticket)
{
    if (!s || !ticket) return fail(LT_ERR_INVALID, "null argument");
    return serve_submit(s, source, walkers, seed, arrival_ms, ticket);
}

lt_status lt_serve_step(lt_server *s, uint32_t *completed, uint32_t *active, uint32_t *pending)
{
    if (!s) return fail(LT_ERR_INVALID, "null server");
    return serve_step(s, completed, active, pending);
}

lt_status lt_serve_result(lt_server *s, uint64_t ticket, int *done, uint64_t *n_pairs, uint32_t *vertices,
                          uint32_t *counts, uint64_t capacity, double *latency_ms)
{
    if (!s) return fail(LT_ERR_INVALID, "null server");
    return serve_result(s, ticket, done, n_pairs, vertices, counts, capacity, latency_ms);
}

uint64_t lt_serve_finished(lt_server *s, uint64_t *tickets, uint64_t cap)
{
    return s ? serve_finished(s, tickets, cap) : 0;
}

void lt_serve_close(lt_server *s) { serve_close(s); }

double lt_serve_now_ms(void) { return serve_now_ms(); }

lt_status lt_engine_autotune(lt_engine *e)
{
    if (!e) return fail(LT_ERR_INVALID, "null engine");
    if (e->ooc) {
        LT_CUDA_TRY(cudaSetDevice(e->device));
        return ooc_autotune(e, &e->ooc_tune);
    }
    return batch_autotune(e);
}

lt_status lt_engine_ooc_tune(const lt_engine *e, lt_ooc_tune *out)
{
    if (!e || !out) return fail(LT_ERR_INVALID, "null argument");
    *out = e->ooc_tune;
    return LT_OK;
}

lt_status lt_engine_batch_tune(const lt_engine *e, lt_batch_tune *out)
{
    if (!e || !out) return fail(LT_ERR_INVALID, "null argument");
    const BatchTune t = batch_tune(e);
    out->block = t.block;
    out->ctas_per_sm = t.ctas_per_sm;
    out->load_shift = t.load_shift;
    out->tuned = t.tuned ? 1 : 0;
    return LT_OK;
}

lt_status lt_walk_device(int app, int start_mode, const uint64_t *d_rowptr, const uint32_t *d_col, uint32_t num_nodes,
                         uint32_t source, uint64_t num_walkers, uint32_t length, float prob, uint32_t run,
                         uint64_t seed, uint64_t *d_counts, uint32_t *d_endpoints, uint32_t *d_paths,
                         void *d_scratch, uint64_t *d_stats, void *stream)
{
    return walk_device(app, start_mode, d_rowptr, d_col, num_nodes, source, num_walkers, length, prob, run, seed,
                       d_counts, d_endpoints, d_paths, d_scratch, d_stats, (cudaStream_t)stream, 0);
}

lt_status lt_walk_device_compact(int app, int start_mode, const uint32_t *d_rowptr32, const uint32_t *d_col,
                                 uint32_t num_nodes, uint32_t source, uint64_t num_walkers, uint32_t length,
                                 float prob, uint32_t run, uint64_t seed, uint32_t *d_counts32,
                                 uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch, uint64_t *d_stats,
                                 void *stream)
{
    return walk_device_compact(app, start_mode, d_rowptr32, d_col, num_nodes, source, num_walkers, length, prob, run,
                               seed, d_counts32, d_endpoints, d_paths, d_scratch, d_stats, (cudaStream_t)stream, 0);
}

lt_status lt_walk_device_packed(int app, int start_mode, uint32_t *d_rows, const uint32_t *d_col, uint32_t num_nodes,
                                uint32_t source, uint64_t num_walkers, uint32_t length, float prob, uint32_t run,
                                uint64_t seed, uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch,
                                uint64_t *d_stats, void *stream)
{
    return walk_device_packed(app, start_mode, d_rows, d_col, num_nodes, source, num_walkers, length, prob, run, seed,
                              d_endpoints, d_paths, d_scratch, d_stats, (cudaStream_t)stream, 0);
}

lt_status lt_rows_pack(const uint64_t *d_rowptr, uint32_t *d_rows, uint32_t num_nodes, void *stream)
{
    return rows_pack(d_rowptr, d_rows, num_nodes, (cudaStream_t)stream);
}

lt_status lt_rows_counts(const uint32_t *d_rows, uint64_t *d_counts, uint32_t num_nodes, void *stream)
{
    return rows_counts(d_rows, d_counts, num_nodes, (cudaStream_t)stream);
}

lt_status lt_engine_checkpoint(lt_engine *e, const char *path, uint64_t every, int stop)
{
    if (!e) return fail(LT_ERR_INVALID, "null engine");
    if (!e->ooc) return fail(LT_ERR_UNSUPPORTED, "checkpoints apply to out-of-core engines (-p below the partition count)");
    if (path && every == 0) return fail(LT_ERR_INVALID, "checkpoint interval must be positive");
    return ooc_checkpoint(e->ooc, path, every, stop);
}

lt_status lt_checkpoint_read_info(const char *path, lt_checkpoint_info *out)
{
    if (!path || !out) return fail(LT_ERR_INVALID, "null argument");
    return checkpoint_info(path, out);
}

lt_status lt_resume(lt_engine *e, const char *path, uint64_t *counts_out, uint32_t *endpoints_out, uint32_t *paths_out)
{
    if (!e || !path) return fail(LT_ERR_INVALID, "null argument");
    if (!e->ooc) return fail(LT_ERR_UNSUPPORTED, "checkpoints apply to out-of-core engines (-p below the partition count)");
    LT_CUDA_TRY(cudaSetDevice(e->device));
    return ooc_resume(e, path, counts_out, endpoints_out, paths_out);
}

lt_status lt_host_alloc(uint64_t bytes, void **out)
{
    if (!out) return fail(LT_ERR_INVALID, "null output");
    *out = nullptr;
    void *p = nullptr;
    const cudaError_t ce = cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocPortable | cudaHostAllocMapped);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return fail(ce == cudaErrorMemoryAllocation ? LT_ERR_NOMEM : LT_ERR_CUDA, "cudaHostAlloc of %llu bytes: %s",
                    (unsigned long long)bytes, cudaGetErrorString(ce));
    }
    *out = p;
    return LT_OK;
}

void lt_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}

lt_status lt_rowptr_narrow(const uint64_t *d_rowptr, uint32_t *d_rowptr32, uint32_t num_nodes, void *stream)
{
    return rowptr_narrow(d_rowptr, d_rowptr32, num_nodes, (cudaStream_t)stream);
}

lt_status lt_abi_field(const char *type, const char *field, size_t *offset, size_t *size)
{
    if (!type || !field || !offset || !size) return LT_ERR_INVALID;
    for (const AbiField &f : kAbiFields)
        if (std::strcmp(f.type, type) == 0 && std::strcmp(f.field, field) == 0) {
            *offset = f.offset;
            *size = f.size;
            return LT_OK;
        }
    return LT_ERR_INVALID;
}

size_t lt_abi_sizeof(const char *type)
{
    if (!type) return 0;
    for (const auto &t : kAbiTypes)
        if (std::strcmp(t.type, type) == 0) return t.size;
    return 0;
}

}  // extern "C"
