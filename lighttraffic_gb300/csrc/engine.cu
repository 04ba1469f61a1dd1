// engine.cu -- engine state, partition cache and the run loop.
//
// Replaces the GPU/CPU device objects and the Scheduler's run loop
// (src/Device.h:7-59, src/LightTraffic.h:33-44, src/Scheduler.h:425-438).
#include "engine.h"

#include <algorithm>
#include <cstring>

#include "lt_core.cuh"
#include "walk_whole.h"

namespace lt {

namespace {

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

lt_status grow(void **p, uint64_t &cap, uint64_t need_bytes)
{
    if (cap >= need_bytes && *p) return LT_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = 0;
    if (cudaMalloc(p, need_bytes ? need_bytes : 4) != cudaSuccess) {
        cudaGetLastError();
        return fail(LT_ERR_NOMEM, "cudaMalloc of %llu bytes failed", (unsigned long long)need_bytes);
    }
    cap = need_bytes;
    return LT_OK;
}

// Scratch layout of the resident step kernel: the next-walker counter.
constexpr size_t kScratchBytes = 256;

}  // namespace

size_t walk_scratch_bytes() { return kScratchBytes; }

namespace {

__global__ void narrow_kernel(uint32_t *dst, const uint64_t *src, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = (uint32_t)src[i];
}

__global__ void widen_kernel(uint64_t *dst, const uint32_t *src, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

unsigned stream_blocks(uint64_t n, int sms) { return (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8); }

// Counter updates of one launch: one per walk (PPR), one per step (PageRank).
uint64_t count_updates(int app, uint64_t W, uint32_t length)
{
    if (app == kPPR) return W;
    if (app == kPageRank) return length && W > UINT64_MAX / length ? UINT64_MAX : W * length;
    return 0;
}

// One launch of the resident step kernel, standard (u64 row offsets and
// counters) or compact (u32, when d_rowptr32 is given).
lt_status walk_launch(int app, int start, const uint64_t *d_rowptr, const uint32_t *d_rowptr32, const uint32_t *d_col,
                      uint32_t V, uint32_t source, uint64_t W, uint32_t length, float prob, uint32_t run,
                      uint64_t seed, uint64_t *d_counts, uint32_t *d_counts32, uint32_t *d_endpoints,
                      uint32_t *d_paths, void *d_scratch, uint64_t *d_stats, cudaStream_t st, int ctas_per_sm,
                      uint32_t *d_rows = nullptr)
{
    const int layout = d_rows ? kLayoutPacked : d_rowptr32 ? kLayoutCompact : kLayoutWide;
    if (app < kPPR || app > kWalk) return fail(LT_ERR_INVALID, "unknown app %d", app);
    if (start < kStartSource || start > kStartPerVertex) return fail(LT_ERR_INVALID, "unknown start mode %d", start);
    if ((layout == kLayoutWide && !d_rowptr) || !d_col || V == 0) return fail(LT_ERR_INVALID, "empty graph");
    if (!d_scratch) return fail(LT_ERR_INVALID, "scratch buffer is required");
    if (app != kWalk && layout == kLayoutWide && !d_counts)
        return fail(LT_ERR_INVALID, "counts buffer is required for PPR and PageRank");
    if (app != kWalk && layout == kLayoutCompact && !d_counts32)
        return fail(LT_ERR_INVALID, "counts buffer is required for PPR and PageRank");
    if (app == kPPR && !(prob > 0.0f && prob <= 1.0f)) return fail(LT_ERR_INVALID, "PPR stop probability must be in (0, 1]");
    if (app != kPPR && length == 0) return fail(LT_ERR_INVALID, "walk length must be positive");
    if (start == kStartSource && source >= V) return fail(LT_ERR_INVALID, "source %u out of range (V=%u)", source, V);
    if (run > 0xFFFFFFu) return fail(LT_ERR_INVALID, "run index %u exceeds 2^24 - 1", run);
    if (app != kWalk) d_paths = nullptr;
    if (W == 0) return LT_OK;
    int device = 0;
    LT_CUDA_TRY(cudaGetDevice(&device));
    WholeArgs a{};
    a.rowptr = d_rowptr;
    a.rowptr32 = d_rowptr32;
    a.counts32 = d_counts32;
    a.rows = d_rows;
    a.col = d_col;
    a.V = V;
    a.source = source;
    a.W = W;
    a.length = length;
    a.run = run;
    a.seed = seed;
    a.thr = app == kWalk ? 0 : threshold53(prob);
    a.counts = d_counts;
    a.endpoints = d_endpoints;
    a.paths = d_paths;
    a.next = (uint64_t *)d_scratch;
    a.stats = d_stats;
    LT_CUDA_TRY(cudaMemsetAsync(d_scratch, 0, kScratchBytes, st));
    const int grid = whole_grid(app, start, device, ctas_per_sm, layout);
    LT_CUDA_TRY(launch_walk_whole(a, app, start, grid, st, layout));
    return LT_OK;
}

}  // namespace

lt_status walk_device(int app, int start, const uint64_t *d_rowptr, const uint32_t *d_col, uint32_t V,
                      uint32_t source, uint64_t W, uint32_t length, float prob, uint32_t run, uint64_t seed,
                      uint64_t *d_counts, uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch,
                      uint64_t *d_stats, cudaStream_t st, int ctas_per_sm)
{
    return walk_launch(app, start, d_rowptr, nullptr, d_col, V, source, W, length, prob, run, seed, d_counts, nullptr,
                       d_endpoints, d_paths, d_scratch, d_stats, st, ctas_per_sm);
}

lt_status walk_device_compact(int app, int start, const uint32_t *d_rowptr32, const uint32_t *d_col, uint32_t V,
                              uint32_t source, uint64_t W, uint32_t length, float prob, uint32_t run, uint64_t seed,
                              uint32_t *d_counts32, uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch,
                              uint64_t *d_stats, cudaStream_t st, int ctas_per_sm)
{
    if (!d_rowptr32) return fail(LT_ERR_INVALID, "empty graph");
    if (count_updates(app, W, length) >= (1ull << 32))
        return fail(LT_ERR_INVALID, "%s updates of %llu walkers overflow u32 counters: use lt_walk_device",
                    app == kPPR ? "PPR" : "PageRank", (unsigned long long)W);
    return walk_launch(app, start, nullptr, d_rowptr32, d_col, V, source, W, length, prob, run, seed, nullptr,
                       d_counts32, d_endpoints, d_paths, d_scratch, d_stats, st, ctas_per_sm);
}

lt_status walk_device_packed(int app, int start, uint32_t *d_rows, const uint32_t *d_col, uint32_t V, uint32_t source,
                             uint64_t W, uint32_t length, float prob, uint32_t run, uint64_t seed,
                             uint32_t *d_endpoints, uint32_t *d_paths, void *d_scratch, uint64_t *d_stats,
                             cudaStream_t st, int ctas_per_sm)
{
    if (!d_rows) return fail(LT_ERR_INVALID, "empty graph");
    if (count_updates(app, W, length) >= (1ull << 32))
        return fail(LT_ERR_INVALID, "%s updates of %llu walkers overflow u32 counters: use lt_walk_device",
                    app == kPPR ? "PPR" : "PageRank", (unsigned long long)W);
    return walk_launch(app, start, nullptr, nullptr, d_col, V, source, W, length, prob, run, seed, nullptr, nullptr,
                       d_endpoints, d_paths, d_scratch, d_stats, st, ctas_per_sm, d_rows);
}

namespace {
__global__ void pack_kernel(uint32_t *rows, const uint64_t *rowptr, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        rows[2 * i] = (uint32_t)rowptr[i];
        rows[2 * i + 1] = 0;
    }
}

__global__ void rows_counts_kernel(uint64_t *counts, const uint32_t *rows, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) counts[i] = rows[2 * i + 1];
}
}  // namespace

lt_status rows_pack(const uint64_t *d_rowptr, uint32_t *d_rows, uint32_t V, cudaStream_t st)
{
    if (!d_rowptr || !d_rows) return fail(LT_ERR_INVALID, "null buffer");
    int device = 0, sms = 0;
    LT_CUDA_TRY(cudaGetDevice(&device));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const uint64_t n = (uint64_t)V + 1;
    pack_kernel<<<stream_blocks(n, sms), 256, 0, st>>>(d_rows, d_rowptr, n);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

lt_status rows_counts(const uint32_t *d_rows, uint64_t *d_counts, uint32_t V, cudaStream_t st)
{
    if (!d_rows || !d_counts) return fail(LT_ERR_INVALID, "null buffer");
    int device = 0, sms = 0;
    LT_CUDA_TRY(cudaGetDevice(&device));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    rows_counts_kernel<<<stream_blocks(V, sms), 256, 0, st>>>(d_counts, d_rows, V);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

lt_status rowptr_narrow(const uint64_t *d_rowptr, uint32_t *d_rowptr32, uint32_t V, cudaStream_t st)
{
    if (!d_rowptr || !d_rowptr32) return fail(LT_ERR_INVALID, "null buffer");
    int device = 0, sms = 0;
    LT_CUDA_TRY(cudaGetDevice(&device));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const uint64_t n = (uint64_t)V + 1;
    narrow_kernel<<<stream_blocks(n, sms), 256, 0, st>>>(d_rowptr32, d_rowptr, n);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

lt_status engine_create(lt_graph *g, const lt_engine_cfg &cfg, lt_engine **out)
{
    if (!g || !out) return fail(LT_ERR_INVALID, "null graph or output");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(LT_ERR_CUDA, "no CUDA device is available");
    }
    if (cfg.device < 0 || cfg.device >= ndev) return fail(LT_ERR_INVALID, "device %d out of range", cfg.device);
    lt_engine *e = new lt_engine();
    e->g = g;
    e->cfg = cfg;
    e->device = cfg.device;
    auto bail = [&](lt_status s) {
        engine_destroy(e);
        return s;
    };
    if (cudaSetDevice(e->device) != cudaSuccess) return bail(fail(LT_ERR_CUDA, "cudaSetDevice failed"));
    cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, e->device);
    const uint32_t P = g->P();
    const uint32_t cache = cfg.num_device_partitions == 0 ? P : std::min(cfg.num_device_partitions, P);
    e->resident = cache >= P;
    if (cudaStreamCreateWithFlags(&e->s_compute, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&e->s_copy, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&e->s_copyback, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e->ev_k0) != cudaSuccess || cudaEventCreate(&e->ev_k1) != cudaSuccess)
        return bail(fail(LT_ERR_CUDA, "stream / event creation failed"));
    if ((e->resident && (cudaMalloc(&e->d_rowptr, 8ull * ((uint64_t)g->V + 1)) != cudaSuccess ||
                         cudaMalloc(&e->d_col, 4ull * (g->E ? g->E : 1)) != cudaSuccess)) ||
        cudaMalloc(&e->d_counts, 8ull * g->V) != cudaSuccess ||
        cudaMalloc(&e->d_scratch, walk_scratch_bytes()) != cudaSuccess ||
        cudaMalloc(&e->d_stats, 64) != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(LT_ERR_NOMEM, "device allocation for the resident graph failed"));
    }
    // compact layout of the resident graph: u32 row offsets and counters
    if (e->resident && g->E < (1ull << 32)) {
        if (cudaMalloc(&e->d_rowptr32, 4ull * ((uint64_t)g->V + 1)) != cudaSuccess ||
            cudaMalloc(&e->d_counts32, 4ull * g->V) != cudaSuccess) {
            cudaGetLastError();
            return bail(fail(LT_ERR_NOMEM, "device allocation for the compact row offsets failed"));
        }
    }
    if (!e->resident) {
        lt_status s = ooc_create(e, &e->ooc);
        if (s != LT_OK) return bail(s);
    }
    *out = e;
    return LT_OK;
}

void engine_destroy(lt_engine *e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->s_compute) cudaStreamSynchronize(e->s_compute);
    if (e->ooc) ooc_destroy(e->ooc);
    if (e->batch) batch_destroy(e->batch);
    for (void *p : {(void *)e->d_rowptr, (void *)e->d_col, (void *)e->d_counts, e->d_scratch, (void *)e->d_stats,
                    (void *)e->d_endpoints, (void *)e->d_paths, (void *)e->d_rowptr32, (void *)e->d_counts32})
        if (p) cudaFree(p);
    if (e->ev_k0) cudaEventDestroy(e->ev_k0);
    if (e->ev_k1) cudaEventDestroy(e->ev_k1);
    for (cudaStream_t s : {e->s_compute, e->s_copy, e->s_copyback})
        if (s) cudaStreamDestroy(s);
    delete e;
}

lt_status engine_drop_cache(lt_engine *e)
{
    e->loaded = false;
    if (e->ooc) return ooc_drop_cache(e->ooc);
    return LT_OK;
}

namespace {

// GPUGraph::loadAsync (src/GraphLoader.h:193-214) for every partition: the
// rowptr slice and the col slice of each partition are copied on the copy
// stream.  In resident mode the slots sit back to back, so the device copy is
// one contiguous CSR whose rowptr entries keep their global edge offsets.
lt_status load_all(lt_engine *e)
{
    if (e->loaded) return LT_OK;
    lt_graph &g = *e->g;
    cudaEvent_t a, b;
    LT_CUDA_TRY(cudaEventCreate(&a));
    LT_CUDA_TRY(cudaEventCreate(&b));
    LT_CUDA_TRY(cudaEventRecord(a, e->s_copy));
    for (uint32_t p = 0; p < g.P(); p++) {
        const uint64_t n0 = g.node_off[p], n1 = g.node_off[p + 1];
        const uint64_t e0 = g.edge_off[p], e1 = g.edge_off[p + 1];
        LT_CUDA_TRY(cudaMemcpyAsync(e->d_rowptr + n0, g.rowptr() + n0, 8 * (n1 - n0 + 1), cudaMemcpyHostToDevice,
                                    e->s_copy));
        if (e1 > e0)
            LT_CUDA_TRY(cudaMemcpyAsync(e->d_col + e0, g.col() + e0, 4 * (e1 - e0), cudaMemcpyHostToDevice, e->s_copy));
        e->stats.h2d_graph_bytes += 8 * (n1 - n0 + 1) + 4 * (e1 - e0);
        e->stats.partition_loads++;
        e->stats.graph_loading_calls++;
    }
    if (e->d_rowptr32) LT_TRY(rowptr_narrow(e->d_rowptr, e->d_rowptr32, g.V, e->s_copy));
    LT_CUDA_TRY(cudaEventRecord(b, e->s_copy));
    LT_CUDA_TRY(cudaEventSynchronize(b));
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    e->stats.graph_loading_ms += ms;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    e->loaded = true;
    return LT_OK;
}

}  // namespace

lt_status engine_ensure_loaded(lt_engine *e)
{
    if (!e->resident) return LT_OK;
    return load_all(e);
}

lt_status engine_run(lt_engine *e, int app, int start, uint32_t source, uint64_t W, uint32_t length, uint32_t runs,
                     uint32_t run_base, float prob, uint64_t *counts_out, uint32_t *endpoints_out,
                     uint32_t *paths_out)
{
    lt_graph &g = *e->g;
    if (app == kPPR && source >= g.V) return fail(LT_ERR_INVALID, "source %u out of range (V=%u)", source, g.V);
    if (runs == 0) runs = 1;
    LT_CUDA_TRY(cudaSetDevice(e->device));
    if (!e->resident)
        return ooc_run(e, app, start, source, W, length, runs, run_base, prob, counts_out, endpoints_out, paths_out);
    e->stats = lt_stats{};
    const double t0 = now_ms();
    LT_TRY(load_all(e));
    cudaStream_t st = e->s_compute;
    // compact layout while every counter total of the call fits 32 bits
    const uint64_t upd = count_updates(app, W, length);
    const bool compact = e->d_rowptr32 && (upd == 0 || upd <= (((1ull << 32) - 1) / runs));
    if (app != kWalk) {
        if (compact)
            LT_CUDA_TRY(cudaMemsetAsync(e->d_counts32, 0, 4ull * g.V, st));
        else
            LT_CUDA_TRY(cudaMemsetAsync(e->d_counts, 0, 8ull * g.V, st));
    }
    LT_CUDA_TRY(cudaMemsetAsync(e->d_stats, 0, 64, st));
    if (endpoints_out) LT_TRY(grow((void **)&e->d_endpoints, e->endpoints_cap, 4 * W));
    if (paths_out) LT_TRY(grow((void **)&e->d_paths, e->paths_cap, 4 * W * ((uint64_t)length + 1)));
    LT_CUDA_TRY(cudaEventRecord(e->ev_k0, st));
    for (uint32_t r = 0; r < runs; r++) {
        const bool cnt = app != kWalk;
        LT_TRY(walk_launch(app, start, compact ? nullptr : e->d_rowptr, compact ? e->d_rowptr32 : nullptr, e->d_col,
                           g.V, source, W, length, prob, run_base + r, e->cfg.seed,
                           cnt && !compact ? e->d_counts : nullptr, cnt && compact ? e->d_counts32 : nullptr,
                           endpoints_out ? e->d_endpoints : nullptr, paths_out ? e->d_paths : nullptr, e->d_scratch,
                           e->d_stats, st, e->cfg.ctas_per_sm));
        e->stats.kernel_launches++;
        e->stats.computing_calls++;
    }
    if (compact && app != kWalk) {
        widen_kernel<<<stream_blocks(g.V, e->sms), 256, 0, st>>>(e->d_counts, e->d_counts32, g.V);
        LT_CUDA_TRY(cudaGetLastError());
        e->stats.kernel_launches++;
    }
    LT_CUDA_TRY(cudaEventRecord(e->ev_k1, st));
    if (counts_out) LT_CUDA_TRY(cudaMemcpyAsync(counts_out, e->d_counts, 8ull * g.V, cudaMemcpyDeviceToHost, st));
    if (endpoints_out) LT_CUDA_TRY(cudaMemcpyAsync(endpoints_out, e->d_endpoints, 4 * W, cudaMemcpyDeviceToHost, st));
    if (paths_out)
        LT_CUDA_TRY(cudaMemcpyAsync(paths_out, e->d_paths, 4 * W * ((uint64_t)length + 1), cudaMemcpyDeviceToHost, st));
    uint64_t hs[3] = {0, 0, 0};
    LT_CUDA_TRY(cudaMemcpyAsync(hs, e->d_stats, sizeof hs, cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaStreamSynchronize(st));
    float kms = 0;
    cudaEventElapsedTime(&kms, e->ev_k0, e->ev_k1);
    e->stats.updates = hs[0];
    e->stats.moves = hs[1];
    e->stats.teleports = hs[2];
    e->stats.iterations = 1;
    e->stats.explicit_iterations = 1;
    e->stats.step_kernel_ms = kms;
    e->stats.computing_ms = kms;
    e->stats.running_ms = now_ms() - t0;
    return LT_OK;
}

}  // namespace lt
