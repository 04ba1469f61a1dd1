// ooc.cu -- out-of-core run loop.
//
// Reference loop (plain, FIFO), one iteration per partition
// (GPUScheduler::run, src/Scheduler.h:311-330):
//   1. the policy picks partition p;
//   2. p is made readable: loaded into a cache slot (evicting the policy's
//      victim) or, below the zero-copy threshold, read from pinned host memory
//      over the host link (zeroCopyCompute, :254-273);
//   3. p's spilled walkers come back from the host (walkerLoadingPhase,
//      :215-233), evicting other partitions' walkers to the host if the
//      device pool is short (handleWalkerPoolOverflow, :59-82);
//   4. one step-kernel launch drains p's queue (and creates the walkers that
//      start in p), walking every walker through all readable partitions;
//   5. walkers that leave for an unreadable partition are bucketed into their
//      destination queues by the scatter kernel, into chunks allocated here.
// Wave runs (learned, frequency, batched; wave_step) drain every cached queue
// per launch while the next loads stream in -- see the comment at wave_step.
// Queue bookkeeping lives on the host (exact counts, no per-decision D2H of
// queue metadata as in src/buffer/Pool.h:604-606); per iteration one small
// D2H (the destination histogram) crosses the link, and the work list and
// chunk plan go up by a kernel reading mapped pinned memory.  Checkpoints and
// resume of runs, and the serving loop, are at the end of the file.
#include "ooc.h"

#include <algorithm>
#include <deque>
#include <map>
#include <chrono>
#include <cstring>
#include <cstdio>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "engine.h"
#include "lt_core.cuh"
#include "mlp.h"
#include "walk_part.h"

namespace lt {

uint64_t Queue::dev_count() const
{
    return dev_chunks.empty() ? 0 : (uint64_t)(dev_chunks.size() - 1) * kChunk + tail_fill;
}
uint64_t Queue::host_count() const { return (uint64_t)host_chunks.size() * kChunk; }

namespace {

constexpr uint32_t kHostSlabChunks = 32;  // chunks per pinned host slab (3 MiB)
constexpr uint32_t kNoPart = 0xFFFFFFFFu;

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
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

enum TimerKind { kTGraph = 0, kTCompute = 1, kTZero = 2, kTBucket = 3 };

// Host-link bytes per zero-copy hop: measured with ncu (sectors the
// system-memory L2 filled from host memory) on the 2^33-edge graph, 0.244 of
// the 256 bytes two 128-byte lines per hop would take -- hops grouped by
// partition share lines.  With the vertex index on the device a hop reads
// only its col entry from the host: one 32-byte sector (measured 31.9).
constexpr uint64_t kZeroCopyBytesPerHop = 62;
constexpr uint64_t kZeroCopyBytesPerHopIndexed = 32;

}  // namespace

struct Ooc {
    lt_engine *e = nullptr;
    lt_graph *g = nullptr;
    uint32_t P = 0, K = 0;
    uint64_t slot_stride = 0;
    uint8_t *d_slots = nullptr;
    std::vector<int32_t> slot_of, part_in_slot;
    std::vector<uint64_t> last_used, loaded_at;
    std::vector<unsigned long long> h_rp, h_col;

    uint32_t *d_node_off = nullptr;
    uint64_t *d_edge_off = nullptr;
    unsigned long long *d_rp = nullptr, *d_col = nullptr;

    uint8_t *d_arena = nullptr;
    uint32_t n_chunks = 0;
    std::vector<uint32_t> free_chunks;

    std::vector<HostBuf> host_slabs;
    std::vector<uint32_t> host_free;

    uint64_t staging_cap = 0;
    uint32_t *d_out = nullptr;      // 5 arrays of staging_cap: cur, step, idx, dest, query
    lt_server *serve = nullptr;  // serving state when queries are being served
    uint32_t *d_ctl = nullptr;      // hist[P] | visits[P] | pad | out_n | next | next2 (u64) | bucket_err (u32) | pad
    uint64_t ctl_words = 0;         // u32 words of d_ctl
    uint32_t *d_planbuf = nullptr;  // cursor[P] | win_off[P] | plan chunks
    uint64_t plan_cap = 0;
    uint32_t *d_work = nullptr;
    uint64_t *d_work_off = nullptr;
    uint64_t work_cap = 0;
    unsigned long long *d_stats = nullptr;

    HostBuf h_ctl;   // pinned mirror of d_ctl
    HostBuf h_plan;  // pinned plan block
    HostBuf h_work;  // pinned work list
    // device views of h_plan / h_work (null: not mapped, upload by copy)
    uint8_t *h_plan_dev = nullptr, *h_work_dev = nullptr;
    // inputs of the device-side plan (tail chunk[P] | tail fill[P] | free
    // stack), two halves used by alternate passes: a pass's plan kernel may
    // still be queued while the host writes the next pass's inputs
    HostBuf h_planin;
    uint8_t *h_planin_dev = nullptr;
    uint64_t planin_words = 0;  // words of one half
    uint64_t plan_passes = 0;
    cudaEvent_t ev_ctl = nullptr;  // the control block's copy to the host has landed
    cudaEvent_t ev_steps = nullptr;  // the pass's step kernels have ended
    cudaEvent_t ev_pre = nullptr, ev_aux = nullptr;  // split launches: inputs ready / cached kernel done
    cudaStream_t s_aux = nullptr;  // split launches: the cached-queue kernel's stream
    // wave runs: the policy has yet to see the last iteration's histograms;
    // it does while the next step kernel runs (see observe_due_now)
    bool observe_due = false;
    std::vector<uint32_t> arrivals, visits;
    // per partition over the current run: walkers entering it, those that
    // entered while it was cached, and step-kernel launches it was cached for
    std::vector<uint64_t> run_visits, run_cached_visits, run_cached_launches;
    std::vector<uint64_t> waiting, lazy_left, dev_waiting;
    // 1 + the iteration since which a partition's queue has held walkers
    // without a break (0: empty queue)
    std::vector<uint64_t> wait_since;

    std::vector<Queue> q;
    std::unique_ptr<Policy> policy;
    int32_t prev_loaded = -1, prev_computed = -1;
    uint64_t iteration = 0;
    uint64_t zc_threshold = 0;
    unsigned long long zc_rp_base = 0, zc_col_base = 0;  // zero-copy rowptr and col bases
    // vertex index (rowptr, V+1 u64) resident on the device: slots then hold
    // only col slices and zero-copy hops read rowptr here; null: the
    // reference's layout, rowptr slice then col slice in every slot
    uint32_t *d_index = nullptr;
    // hot-vertex tier (cfg.hot_tier > 0): the adjacency of the vertices read
    // most per byte in the partitions outside the cache, chosen from the
    // counts of the engine's previous run of the same walk, in a device
    // region paid from the -p budget (fewer slots):
    //   uint2 words[ceil(V / 32)] | u32 rank -> pool offset[hot] | u32 pool
    // packed on the host, copied in and marked in the vertex index at a
    // run's start, unmarked when the cache is dropped
    uint64_t tier_bytes = 0;  // device budget, 0 = no tier
    uint8_t *d_tier = nullptr;
    HostBuf h_tier;
    uint64_t tier_words = 0;                 // ceil(V / 32)
    uint64_t tier_hot = 0, tier_used = 0;    // current build: hot vertices, bytes in use
    uint64_t tier_off_at = 0, tier_pool_at = 0;
    bool tier_built = false, tier_loaded = false, tier_ready = false;
    int tier_app = -1, tier_start = -1;
    uint32_t tier_source = 0;
    double tier_build_ms = 0;
    cudaEvent_t ev_tier = nullptr;
    // zero-copy set of the next step kernel (wave runs)
    uint32_t zc_mask[kZcMaskWords] = {};
    bool zc_mask_any = false;
    // checkpoints of runs (lt_engine_checkpoint): every ckpt_every
    // iterations, the run stopping after the first one when ckpt_stop
    std::string ckpt_path;
    uint64_t ckpt_every = 0;
    bool ckpt_stop = false;
    uint32_t run_runs = 1, run_base = 0, run_index = 0;  // multi-run position of the run in progress
    float run_prob = 0.f;
    int grid[3] = {0, 0, 0};

    std::vector<cudaEvent_t> ev_free;
    struct Timed {
        cudaEvent_t a, b;
        int kind;
    };
    std::vector<Timed> timed;

    uint8_t *host_chunk(uint32_t id)
    {
        return (uint8_t *)host_slabs[id / kHostSlabChunks].ptr + (uint64_t)(id % kHostSlabChunks) * kChunkBytes;
    }
    uint32_t hist_words() const { return (2 * P + 1) & ~1u; }
    uint32_t *ctl_hist() { return d_ctl; }
    uint32_t *ctl_visits() { return d_ctl + P; }
    unsigned long long *ctl_out_n() { return (unsigned long long *)(d_ctl + hist_words()); }
    unsigned long long *ctl_next() { return ctl_out_n() + 1; }
    unsigned long long *ctl_next2() { return ctl_out_n() + 2; }  // the second kernel of a split launch
    // set by the bucketing kernel, kept across iterations (not cleared with the rest)
    uint32_t bucket_err_word() const { return hist_words() + 6; }
    uint32_t *ctl_bucket_err() { return d_ctl + bucket_err_word(); }
    uint32_t cleared_words() const { return hist_words() + 6; }
};

namespace {

cudaEvent_t ev_get(Ooc &o)
{
    if (o.ev_free.empty()) {
        cudaEvent_t ev;
        cudaEventCreate(&ev);
        return ev;
    }
    cudaEvent_t ev = o.ev_free.back();
    o.ev_free.pop_back();
    return ev;
}

// Resolve the event timers of finished work into the phase timers.
void drain_timers(Ooc &o, bool all)
{
    lt_engine &e = *o.e;
    // every iteration records a few timers: read them in batches (each read
    // is a few driver calls), and all of them at the end of a run
    if (!all && o.timed.size() < 48) return;
    size_t keep = 0;
    for (size_t i = 0; i < o.timed.size(); i++) {
        Ooc::Timed &t = o.timed[i];
        if (!all && cudaEventQuery(t.b) != cudaSuccess) {
            cudaGetLastError();
            o.timed[keep++] = t;
            continue;
        }
        float ms = 0;
        cudaEventSynchronize(t.b);
        cudaEventElapsedTime(&ms, t.a, t.b);
        if (t.kind == kTGraph)
            e.stats.graph_loading_ms += ms;
        else if (t.kind == kTCompute)
            e.stats.computing_ms += ms;
        else if (t.kind == kTZero)
            e.stats.zerocopy_ms += ms;
        else
            e.stats.bucket_ms += ms;
        if (t.kind == kTCompute || t.kind == kTZero) e.stats.step_kernel_ms += ms;
        o.ev_free.push_back(t.a);
        o.ev_free.push_back(t.b);
    }
    o.timed.resize(keep);
}

// Bytes a load of partition p copies (and its host footprint): the col
// slice with the vertex index resident, else rowptr and col slices.
uint64_t host_part_bytes(const Ooc &o, uint32_t p)
{
    const lt_graph &g = *o.g;
    return o.d_index ? 4 * (g.edge_off[p + 1] - g.edge_off[p]) : g.slot_bytes(p);
}

uint64_t zc_bytes_per_hop(const Ooc &o) { return o.d_index ? kZeroCopyBytesPerHopIndexed : kZeroCopyBytesPerHop; }

__global__ void set_entry_kernel(unsigned long long *rp, unsigned long long *col, uint32_t p, unsigned long long rv,
                                 unsigned long long cv)
{
    rp[p] = rv;
    col[p] = cv;
}

// Table updates travel as kernel arguments, so they are ordered on `st` with
// the kernels that read the table and capture the values at call time.
lt_status set_entry(Ooc &o, uint32_t p, cudaStream_t st)
{
    set_entry_kernel<<<1, 1, 0, st>>>(o.d_rp, o.d_col, p, o.h_rp[p], o.h_col[p]);
    LT_CUDA_TRY(cudaGetLastError());
    o.e->stats.kernel_launches++;
    return LT_OK;
}

__global__ void upload_kernel(uint32_t *dst, const uint32_t *src, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

// Copy `words` u32 words at h_src (inside the pinned buffer hb, whose device
// view is hb_dev) to d_dst on the compute stream.  A kernel reading the mapped
// host buffer does it: an H2D copy on the compute stream would wait on the
// copy engine behind the partition loads queued on the copy stream.
lt_status upload(Ooc &o, void *d_dst, const HostBuf &hb, uint8_t *hb_dev, const void *h_src, uint64_t words)
{
    lt_engine &e = *o.e;
    if (words == 0) return LT_OK;
    if (!hb_dev) {
        LT_CUDA_TRY(cudaMemcpyAsync(d_dst, h_src, 4 * words, cudaMemcpyHostToDevice, e.s_compute));
        return LT_OK;
    }
    const uint32_t *src = (const uint32_t *)(hb_dev + ((const uint8_t *)h_src - (const uint8_t *)hb.ptr));
    const uint64_t blocks = std::min<uint64_t>((words + 255) / 256, 304);
    upload_kernel<<<(unsigned)blocks, 256, 0, e.s_compute>>>((uint32_t *)d_dst, src, words);
    LT_CUDA_TRY(cudaGetLastError());
    e.stats.kernel_launches++;
    return LT_OK;
}

// waiting[] is kept current by refresh() wherever a queue changes.
// ---- hot-vertex tier

// Sets (set) or clears the tier mark (bit 31) in the vertex index entry of
// every vertex the tier's words mark.
__global__ void tier_mark_kernel(uint32_t *index, const uint2 *words, uint64_t n_words, uint32_t V, int set)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_words; w += stride) {
        uint32_t m = words[w].x;
        while (m) {
            const uint32_t b = (uint32_t)__ffs(m) - 1;
            m &= m - 1;
            const uint64_t v = w * 32 + b;
            if (v < V) index[v] = set ? (index[v] | kHotMark) : (index[v] & ~kHotMark);
        }
    }
}

lt_status tier_mark(Ooc &o, int set, cudaStream_t st)
{
    const uint64_t blocks = std::min<uint64_t>((o.tier_words + 255) / 256, 1024);
    tier_mark_kernel<<<(unsigned)blocks, 256, 0, st>>>(o.d_index, (const uint2 *)o.d_tier, o.tier_words, o.g->V, set);
    LT_CUDA_TRY(cudaGetLastError());
    o.e->stats.kernel_launches++;
    return LT_OK;
}

// Copies the built tier in and marks its vertices (copy stream); the step
// kernels use it once the copy has landed (tier_ready, set by wave_step).
lt_status tier_load(Ooc &o)
{
    lt_engine &e = *o.e;
    if (!o.tier_built || o.tier_loaded) return LT_OK;
    LT_CUDA_TRY(cudaMemcpyAsync(o.d_tier, o.h_tier.ptr, o.tier_used, cudaMemcpyHostToDevice, e.s_copy));
    LT_TRY(tier_mark(o, 1, e.s_copy));
    LT_CUDA_TRY(cudaEventRecord(o.ev_tier, e.s_copy));
    e.stats.h2d_graph_bytes += o.tier_used;
    o.tier_loaded = true;
    o.tier_ready = false;
    return LT_OK;
}

// Takes the tier out of use: unmarks the index (after every kernel that may
// read it).
lt_status tier_unload(Ooc &o)
{
    lt_engine &e = *o.e;
    if (!o.tier_loaded) return LT_OK;
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_copy));
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    LT_TRY(tier_mark(o, 0, e.s_compute));
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    o.tier_loaded = o.tier_ready = false;
    return LT_OK;
}

// Builds the tier for the next runs of the same walk from this run's
// per-vertex counts (PPR endpoints, PageRank visits: proportional to the
// reads of each vertex's adjacency).  Candidates are the vertices of the
// partitions outside the cache at the end of the run; each is worth
// counts / (4 deg + 4) (its adjacency and its pool offset), and the best go
// in until the budget is spent: a histogram of the worths (the top 16 bits of
// the float) finds the threshold.
lt_status tier_build(Ooc &o, int app, int start, uint32_t source, const uint64_t *counts)
{
    lt_graph &g = *o.g;
    const double t0 = now_ms();
    LT_TRY(tier_unload(o));
    o.tier_built = false;
    const uint64_t *rowptr = g.rowptr();
    const uint32_t *colp = g.col();
    const uint64_t words_bytes = 8 * o.tier_words;
    const uint64_t budget = o.tier_bytes - words_bytes - 16;
    auto key_of = [&](uint32_t v, uint32_t p) -> int32_t {
        if (o.slot_of[p] >= 0 || counts[v] == 0) return -1;
        const uint64_t deg = rowptr[v + 1] - rowptr[v];
        if (deg == 0) return -1;
        const float worth = (float)counts[v] / (float)(4 * deg + 4);
        uint32_t bits;
        std::memcpy(&bits, &worth, 4);
        return (int32_t)(bits >> 16);
    };
    // histogram of candidate bytes per worth key
    std::vector<uint64_t> hist(1 << 16, 0);
#pragma omp parallel
    {
        std::vector<uint64_t> mine(1 << 16, 0);
#pragma omp for schedule(dynamic, 1)
        for (int64_t p = 0; p < (int64_t)o.P; p++)
            for (uint32_t v = g.node_off[p]; v < g.node_off[p + 1]; v++) {
                const int32_t k = key_of(v, (uint32_t)p);
                if (k >= 0) mine[k] += 4 * (rowptr[v + 1] - rowptr[v]) + 4;
            }
#pragma omp critical
        for (size_t k = 0; k < mine.size(); k++) hist[k] += mine[k];
    }
    int32_t thr = (1 << 16) - 1;
    uint64_t above = 0;
    while (thr >= 0 && above + hist[thr] <= budget) above += hist[thr--];
    // the vertices above the threshold key go in (a key spans under 1 % of
    // worth: the threshold's own key is left out)
    uint2 *words = (uint2 *)o.h_tier.ptr;
    std::memset(words, 0, words_bytes);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t p = 0; p < (int64_t)o.P; p++)
        for (uint32_t v = g.node_off[p]; v < g.node_off[p + 1]; v++)
            if (key_of(v, (uint32_t)p) > thr) __atomic_fetch_or(&words[v >> 5].x, 1u << (v & 31), __ATOMIC_RELAXED);
    // ranks, pool offsets and the pool
    uint64_t hot = 0;
    for (uint64_t w = 0; w < o.tier_words; w++) {
        words[w].y = (uint32_t)hot;
        hot += (uint64_t)__builtin_popcount(words[w].x);
    }
    o.tier_off_at = words_bytes;
    o.tier_pool_at = (o.tier_off_at + 4 * hot + 15) & ~15ull;
    uint32_t *off = (uint32_t *)((uint8_t *)o.h_tier.ptr + o.tier_off_at);
    uint32_t *pool = (uint32_t *)((uint8_t *)o.h_tier.ptr + o.tier_pool_at);
    uint64_t pw = 0;
    for (uint64_t w = 0; w < o.tier_words; w++)
        for (uint32_t m = words[w].x; m; m &= m - 1) {
            const uint64_t v = w * 32 + (uint32_t)__builtin_ctz(m);
            off[words[w].y + (uint32_t)__builtin_popcount(words[w].x & ((1u << (v & 31)) - 1u))] = (uint32_t)pw;
            pw += rowptr[v + 1] - rowptr[v];
        }
    if (o.tier_pool_at + 4 * pw > o.tier_bytes || pw >= (1ull << 32))
        return fail(LT_ERR_CAPACITY, "hot-vertex tier overflows its budget");
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t w = 0; w < (int64_t)o.tier_words; w++)
        for (uint32_t m = words[w].x; m; m &= m - 1) {
            const uint64_t v = (uint64_t)w * 32 + (uint32_t)__builtin_ctz(m);
            const uint32_t r = words[w].y + (uint32_t)__builtin_popcount(words[w].x & ((1u << (v & 31)) - 1u));
            std::memcpy(pool + off[r], colp + rowptr[v], 4 * (rowptr[v + 1] - rowptr[v]));
        }
    o.tier_hot = hot;
    o.tier_used = o.tier_pool_at + 4 * pw;
    o.tier_app = app;
    o.tier_start = start;
    o.tier_source = source;
    o.tier_built = hot > 0;
    o.tier_build_ms = now_ms() - t0;
    return LT_OK;
}

void refresh(Ooc &o, uint32_t p)
{
    o.waiting[p] = o.q[p].total();
    if (o.waiting[p] == 0)
        o.wait_since[p] = 0;
    else if (o.wait_since[p] == 0)
        o.wait_since[p] = o.iteration + 1;
    o.lazy_left[p] = o.q[p].lazy_left();
    o.dev_waiting[p] = o.q[p].dev_count();
}
void refresh_all(Ooc &o)
{
    for (uint32_t p = 0; p < o.P; p++) refresh(o, p);
}

SchedView view(Ooc &o);

// The timers and the policy's per-iteration update of a wave run, deferred
// from the end of an iteration to the moment the next step kernel has been
// submitted, so that they overlap it instead of delaying it: the policy's
// view then lags one iteration behind the queues.
void observe_due_now(Ooc &o)
{
    if (!o.observe_due) return;
    o.observe_due = false;
    const double t0 = now_ms();
    drain_timers(o, false);
    o.policy->observe(view(o));
    o.e->stats.host_observe_ms += now_ms() - t0;
}

SchedView view(Ooc &o)
{
    SchedView v;
    v.P = o.P;
    v.K = o.K;
    v.waiting = o.waiting.data();
    v.lazy = o.lazy_left.data();
    v.dev = o.dev_waiting.data();
    v.slot_of = o.slot_of.data();
    v.last_used = o.last_used.data();
    v.arrivals = o.arrivals.data();
    v.visits = o.visits.data();
    v.iteration = o.iteration;
    v.zc_threshold = o.zc_threshold;
    return v;
}

// Table entry of a partition outside the cache: unreadable (zero-copy reads
// go through the per-launch zc_part / zc_mask instead).
void uncached_entry(Ooc &o, uint32_t p)
{
    o.h_rp[p] = 0;
    o.h_col[p] = 0;
}

// Clear v's table entry on the compute stream.  Kernels enqueued before this
// point may still read the slot; loads into the slot wait for this point.

lt_status evict_partition(Ooc &o, uint32_t v)
{
    const int32_t s = o.slot_of[v];
    o.slot_of[v] = -1;
    o.part_in_slot[s] = -1;
    uncached_entry(o, v);
    return set_entry(o, v, o.e->s_compute);
}

int32_t free_slot(Ooc &o)
{
    for (uint32_t s = 0; s < o.K; s++)
        if (o.part_in_slot[s] < 0) return (int32_t)s;
    return -1;
}

// GPUGraph::loadAsync (src/GraphLoader.h:193-214): the rowptr slice, then the
// col slice at the next 16-byte boundary of slot `slot` (only the col slice
// when the vertex index is resident), on the copy stream
// after every compute operation enqueued so far (the slot's previous occupant
// may still be read by them).  The table entry is published on the compute
// stream once the copy is done: right away (the next kernel waits for the
// copy), or, for the loads of a wave, before the next wave's kernel.
lt_status start_load(Ooc &o, uint32_t p, int32_t slot, std::vector<std::pair<uint32_t, cudaEvent_t>> *deferred)
{
    lt_engine &e = *o.e;
    lt_graph &g = *o.g;
    cudaEvent_t free_ev = ev_get(o);
    LT_CUDA_TRY(cudaEventRecord(free_ev, e.s_compute));
    LT_CUDA_TRY(cudaStreamWaitEvent(e.s_copy, free_ev, 0));
    o.ev_free.push_back(free_ev);

    const uint64_t n0 = g.node_off[p], n1 = g.node_off[p + 1];
    const uint64_t e0 = g.edge_off[p], e1 = g.edge_off[p + 1];
    uint8_t *base = o.d_slots + (uint64_t)slot * o.slot_stride;
    const uint64_t rp_bytes = o.d_index ? 0 : 8 * (n1 - n0 + 1);
    const uint64_t col_off = (rp_bytes + 15) & ~15ull;
    Ooc::Timed t{ev_get(o), ev_get(o), kTGraph};
    LT_CUDA_TRY(cudaEventRecord(t.a, e.s_copy));
    if (rp_bytes) LT_CUDA_TRY(cudaMemcpyAsync(base, g.rowptr() + n0, rp_bytes, cudaMemcpyHostToDevice, e.s_copy));
    if (e1 > e0) LT_CUDA_TRY(cudaMemcpyAsync(base + col_off, g.col() + e0, 4 * (e1 - e0), cudaMemcpyHostToDevice, e.s_copy));
    LT_CUDA_TRY(cudaEventRecord(t.b, e.s_copy));
    o.timed.push_back(t);
    o.h_rp[p] = (unsigned long long)(uintptr_t)(o.d_index ? (uint8_t *)(o.d_index + n0) : base);
    o.h_col[p] = (unsigned long long)(uintptr_t)(base + col_off);
    o.loaded_at[p] = o.iteration;
    o.slot_of[p] = slot;
    o.part_in_slot[slot] = (int32_t)p;
    if (deferred) {
        deferred->push_back({p, t.b});
    } else {
        LT_CUDA_TRY(cudaStreamWaitEvent(e.s_compute, t.b, 0));
        LT_TRY(set_entry(o, p, e.s_compute));
    }
    e.stats.graph_loading_calls++;
    e.stats.h2d_graph_bytes += rp_bytes + 4 * (e1 - e0);
    e.stats.partition_loads++;
    return LT_OK;
}

lt_status load_partition(Ooc &o, uint32_t p, std::vector<std::pair<uint32_t, cudaEvent_t>> *deferred)
{
    if (o.slot_of[p] >= 0) return LT_OK;
    int32_t slot = free_slot(o);
    if (slot < 0) {
        SchedView v = view(o);
        int32_t victim = o.policy->victim(v, o.prev_loaded, p);
        // with a single slot the partition loaded last is the only candidate
        // (the reference asserts here, src/Scheduler.h:169)
        if (victim < 0) victim = o.policy->victim(v, -1, p);
        if (victim < 0) return fail(LT_ERR_CAPACITY, "no cached partition can be evicted");
        slot = o.slot_of[victim];
        LT_TRY(evict_partition(o, (uint32_t)victim));
    }
    return start_load(o, p, slot, deferred);
}

lt_status host_chunk_alloc(Ooc &o, uint32_t &id)
{
    if (o.host_free.empty()) {
        HostBuf b;
        LT_TRY(host_alloc(b, kHostSlabChunks * kChunkBytes, true));
        const uint32_t slab = (uint32_t)o.host_slabs.size();
        o.host_slabs.push_back(b);
        for (uint32_t i = kHostSlabChunks; i-- > 0;) o.host_free.push_back(slab * kHostSlabChunks + i);
    }
    id = o.host_free.back();
    o.host_free.pop_back();
    return LT_OK;
}

// Move full device chunks of other partitions to the host until `need` device
// chunks are free (setEvictedWalker / getEvictedPartition, src/Scheduler.h:53-57,
// :130-147: the partition with the fewest walkers among those holding a full
// page on the device).
lt_status spill_until(Ooc &o, uint64_t need, int32_t except)
{
    lt_engine &e = *o.e;
    double t0 = -1;
    while (o.free_chunks.size() < need) {
        int32_t best = -1;
        for (uint32_t i = 0; i < o.P; i++) {
            if ((int32_t)i == except) continue;
            const Queue &qi = o.q[i];
            if (qi.dev_chunks.empty()) continue;
            const size_t full = qi.dev_chunks.size() - (qi.tail_fill == kChunk ? 0 : 1);
            if (full == 0) continue;
            if (best < 0 || qi.total() < o.q[best].total()) best = (int32_t)i;
        }
        if (best < 0)
            return fail(LT_ERR_CAPACITY, "walker pool of %u chunks cannot hold the walkers in flight (-b too small)",
                        o.n_chunks);
        if (t0 < 0) {
            LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
            t0 = now_ms();
        }
        Queue &qb = o.q[best];
        const size_t full = qb.dev_chunks.size() - (qb.tail_fill == kChunk ? 0 : 1);
        size_t moved = 0;
        for (size_t k = 0; k < full && o.free_chunks.size() + moved < need; k++) {
            uint32_t hid;
            LT_TRY(host_chunk_alloc(o, hid));
            const uint32_t dc = qb.dev_chunks[k];
            LT_CUDA_TRY(cudaMemcpyAsync(o.host_chunk(hid), o.d_arena + (uint64_t)dc * kChunkBytes, kChunkBytes,
                                        cudaMemcpyDeviceToHost, e.s_copyback));
            qb.host_chunks.push_back(hid);
            moved++;
            e.stats.d2h_walker_bytes += kChunkBytes;
        }
        for (size_t k = 0; k < moved; k++) o.free_chunks.push_back(qb.dev_chunks[k]);
        qb.dev_chunks.erase(qb.dev_chunks.begin(), qb.dev_chunks.begin() + moved);
        if (qb.dev_chunks.empty()) qb.tail_fill = 0;
        refresh(o, (uint32_t)best);
        e.stats.walker_evicting_calls++;
    }
    if (t0 >= 0) {
        LT_CUDA_TRY(cudaStreamSynchronize(e.s_copyback));
        e.stats.walker_evicting_ms += now_ms() - t0;
    }
    return LT_OK;
}

// Bring up to `max_chunks` of p's spilled chunks back to the device
// (walkerLoadingPhase); they go in front of p's device chunks.
lt_status unspill(Ooc &o, uint32_t p, uint64_t max_chunks)
{
    lt_engine &e = *o.e;
    Queue &qp = o.q[p];
    const uint64_t n = std::min<uint64_t>(max_chunks, qp.host_chunks.size());
    if (n == 0) return LT_OK;
    const double t0 = now_ms();
    std::vector<uint32_t> fresh;
    for (uint64_t k = 0; k < n; k++) {
        const uint32_t hid = qp.host_chunks.back();
        qp.host_chunks.pop_back();
        const uint32_t dc = o.free_chunks.back();
        o.free_chunks.pop_back();
        LT_CUDA_TRY(cudaMemcpyAsync(o.d_arena + (uint64_t)dc * kChunkBytes, o.host_chunk(hid), kChunkBytes,
                                    cudaMemcpyHostToDevice, e.s_copy));
        o.host_free.push_back(hid);
        fresh.push_back(dc);
        e.stats.h2d_walker_bytes += kChunkBytes;
    }
    if (qp.dev_chunks.empty()) qp.tail_fill = kChunk;
    qp.dev_chunks.insert(qp.dev_chunks.begin(), fresh.begin(), fresh.end());
    refresh(o, p);
    // the host slots are reused only after the copy: wait here
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_copy));
    e.stats.walker_loading_ms += now_ms() - t0;
    e.stats.walker_loading_calls++;
    return LT_OK;
}

void serve_args(Ooc &o, StepArgs &a);

struct RunParams {
    int app, start;
    uint32_t source, length, run;
    uint64_t W, thr;
    uint64_t *counts;
    uint32_t *endpoints, *paths;
};

// Launch the step kernel over p's device chunks plus G lazily created walkers
// (ordinals lazy_begin..), then bucket the walkers that left.  p < 0: the
// lazily created walkers have uniform random starts and belong to no
// partition yet (the reference's createWalkers / insert, src/WalkManager.h:341-360).
struct Lazy {
    int mode;           // lt::Start
    uint32_t nb, n;     // per-vertex starts: vertex range
    uint64_t begin, count;
};

Lazy lazy_of(Ooc &o, const RunParams &rp, int32_t p, uint64_t begin, uint64_t count)
{
    Lazy z{};
    z.begin = begin;
    z.count = count;
    if (p < 0) {
        z.mode = rp.start;
        z.nb = 0;
        z.n = o.g->V;
    } else {
        z.mode = rp.start == kStartPerVertex ? kStartPerVertex : kStartSource;
        z.nb = o.g->node_off[p];
        z.n = o.g->node_off[p + 1] - z.nb;
    }
    return z;
}

lt_status step_and_bucket_parts(Ooc &o, const RunParams &rp, const std::vector<uint32_t> &parts, int32_t p,
                                const Lazy &lz, bool zero_copy, std::vector<std::pair<uint32_t, cudaEvent_t>> *deferred);

// Appends h_hist[d] walkers to every destination queue: after the walkers of
// its open tail chunk, then in new chunks popped from the free stack in
// destination order (plan_kernel's arithmetic).  With h_cursor given, also
// writes the pass's plan: per destination its first slot in the window and
// the window's start in h_chunks.  Returns the plan's length.  The caller
// has made sure the free stack holds every chunk needed.
uint64_t plan_windows(Ooc &o, const uint32_t *h_hist, uint32_t *h_cursor, uint32_t *h_win, uint32_t *h_chunks)
{
    uint64_t n_plan = 0;
    for (uint32_t d = 0; d < o.P; d++) {
        if (h_cursor) h_cursor[d] = h_win[d] = 0;
        if (!h_hist[d]) continue;
        Queue &qd = o.q[d];
        if (qd.dev_chunks.empty() || qd.tail_fill == kChunk) {
            qd.dev_chunks.push_back(o.free_chunks.back());
            o.free_chunks.pop_back();
            qd.tail_fill = 0;
        }
        if (h_cursor) {
            h_win[d] = (uint32_t)n_plan;
            h_cursor[d] = qd.tail_fill;
            h_chunks[n_plan] = qd.dev_chunks.back();
        }
        n_plan++;
        const uint64_t tot = (uint64_t)qd.tail_fill + h_hist[d];
        const uint64_t extra = (tot + kChunk - 1) / kChunk - 1;
        for (uint64_t k = 0; k < extra; k++) {
            const uint32_t c = o.free_chunks.back();
            o.free_chunks.pop_back();
            qd.dev_chunks.push_back(c);
            if (h_cursor) h_chunks[n_plan] = c;
            n_plan++;
        }
        qd.tail_fill = (uint32_t)(tot - extra * kChunk);
        refresh(o, d);
    }
    return n_plan;
}

lt_status step_and_bucket(Ooc &o, const RunParams &rp, int32_t p, const Lazy &lz, bool zero_copy,
                          std::vector<std::pair<uint32_t, cudaEvent_t>> *deferred)
{
    std::vector<uint32_t> parts;
    if (p >= 0) parts.push_back((uint32_t)p);
    return step_and_bucket_parts(o, rp, parts, p, lz, zero_copy, deferred);
}

// Drain the queues of `parts` (and create lz.count lazy walkers, belonging to
// partition p when p >= 0) in one step-kernel launch.
lt_status step_and_bucket_parts(Ooc &o, const RunParams &rp, const std::vector<uint32_t> &parts, int32_t p,
                                const Lazy &lz, bool zero_copy, std::vector<std::pair<uint32_t, cudaEvent_t>> *deferred)
{
    const uint64_t G = lz.count;
    lt_engine &e = *o.e;
    lt_graph &g = *o.g;
    const double t_submit = now_ms();
    Queue *qp = p >= 0 ? &o.q[p] : nullptr;
    uint64_t n_chunk_walkers = 0, nw = 0;
    for (uint32_t x : parts) {
        n_chunk_walkers += o.q[x].dev_count();
        nw += o.q[x].dev_chunks.size();
    }
    if (n_chunk_walkers + G == 0) return LT_OK;
    if (n_chunk_walkers + G > o.staging_cap) return fail(LT_ERR_CAPACITY, "staging area too small");
    if (nw > o.work_cap) return fail(LT_ERR_CAPACITY, "work list too small");
    // Split launch (wave runs with a zero-copy group): the walkers of cached
    // queues and those created now run in a kernel of their own on one CTA
    // per SM, the zero-copy group's walkers in a kernel on the rest,
    // concurrently.  A warp advances at the pace of its slowest lane, so
    // walkers that read only device memory, mixed into warps waiting on host
    // reads, would move at the host reads' pace (c2: 0.935 -> 0.909 s and
    // 0.952 -> 0.934 s per run; two CTAs per SM for the cached kernel: 0.973).
    auto in_group = [&](uint32_t x) { return o.zc_mask_any && ((o.zc_mask[x >> 5] >> (x & 31)) & 1u); };
    std::vector<uint32_t> order;
    uint64_t nw_a = 0, walkers_a = 0;  // the cached part of a split launch
    bool split = false;
    if (o.zc_mask_any && !zero_copy && !e.cfg.no_split && o.grid[rp.app] >= 2 * e.sms) {
        for (uint32_t x : parts)
            if (!in_group(x)) {
                order.push_back(x);
                nw_a += o.q[x].dev_chunks.size();
                walkers_a += o.q[x].dev_count();
            }
        for (uint32_t x : parts)
            if (in_group(x)) order.push_back(x);
        split = walkers_a + G > 0 && n_chunk_walkers > walkers_a;
    }
    const std::vector<uint32_t> &lst = split ? order : parts;
    uint32_t *h_work = (uint32_t *)o.h_work.ptr;
    uint64_t *h_woff = (uint64_t *)(h_work + ((o.work_cap + 1) & ~1ull));
    const bool multi = parts.size() > 1 || split;
    {
        uint64_t k = 0, ord = 0;
        for (uint32_t x : lst) {
            const Queue &qx = o.q[x];
            for (size_t c = 0; c < qx.dev_chunks.size(); c++, k++) {
                if (split && k == nw_a) ord = 0;  // the second kernel's ordinals start again
                h_work[k] = qx.dev_chunks[c];
                h_woff[k] = ord;
                ord += c + 1 == qx.dev_chunks.size() ? qx.tail_fill : kChunk;
            }
        }
    }
    if (nw) {
        LT_TRY(upload(o, o.d_work, o.h_work, o.h_work_dev, h_work, nw));
        if (multi) LT_TRY(upload(o, o.d_work_off, o.h_work, o.h_work_dev, h_woff, 2 * nw));
    }
    // Plan the bucketing pass on the device, right behind the step kernel,
    // when the free chunks provably hold every arrival: at most n_in walkers
    // leave, which need at most ceil(n_in / kChunk) chunks plus one per
    // destination.  The drained chunks go back to the pool first (the plan
    // may reuse them once the step kernel has read them).  Otherwise the
    // host plans after reading the histogram (and may spill walkers first).
    const uint64_t n_in = n_chunk_walkers + G;
    const uint64_t need_max = (n_in + kChunk - 1) / kChunk + std::min<uint64_t>(o.P, n_in);
    bool dev_plan = false;
    if (o.P <= kSmemPartMax && o.h_planin_dev && !e.cfg.host_plan) {
        uint64_t free_after = o.free_chunks.size();
        for (uint32_t x : parts) free_after += o.q[x].dev_chunks.size();
        dev_plan = need_max <= free_after && need_max + o.P <= o.plan_cap;
    }
    PlanArgs pa{};
    if (dev_plan) {
        for (uint32_t x : parts) {
            Queue &qx = o.q[x];
            for (uint32_t c : qx.dev_chunks) o.free_chunks.push_back(c);
            qx.dev_chunks.clear();
            qx.tail_fill = 0;
            refresh(o, x);
        }
        const uint64_t half = (o.plan_passes++ & 1) * o.planin_words;
        uint32_t *h_in = (uint32_t *)o.h_planin.ptr + half;
        for (uint32_t d = 0; d < o.P; d++) {
            const Queue &qd = o.q[d];
            h_in[d] = qd.dev_chunks.empty() ? kNoChunk : qd.dev_chunks.back();
            h_in[o.P + d] = qd.tail_fill;
        }
        const uint64_t n_stack = std::min<uint64_t>(need_max, o.free_chunks.size());
        for (uint64_t i = 0; i < n_stack; i++) h_in[2ull * o.P + i] = o.free_chunks[o.free_chunks.size() - 1 - i];
        const uint32_t *d_in = (const uint32_t *)(o.h_planin_dev + 4 * half);
        pa.hist = o.ctl_hist();
        pa.tail_chunk = d_in;
        pa.tail_fill = d_in + o.P;
        pa.stack = d_in + 2ull * o.P;
        pa.n_stack = (uint32_t)n_stack;
        pa.P = o.P;
        pa.cursor = o.d_planbuf;
        pa.win_off = o.d_planbuf + o.P;
        pa.plan_chunks = o.d_planbuf + 2ull * o.P;
        pa.plan_cap = o.plan_cap;
        pa.err = o.ctl_bucket_err();
    }
    LT_CUDA_TRY(cudaMemsetAsync(o.d_ctl, 0, 4ull * o.cleared_words(), e.s_compute));

    StepArgs a{};
    a.t = PartTable{o.d_node_off, o.d_edge_off, o.d_rp, o.d_col, o.P};
    a.arena = o.d_arena;
    a.work_chunks = o.d_work;
    a.n_chunk_walkers = n_chunk_walkers;
    a.work_off = multi && nw ? o.d_work_off : nullptr;
    a.n_work = (uint32_t)nw;
    a.lazy_begin = lz.begin;
    a.lazy_count = G;
    a.lazy_nb = lz.nb;
    a.lazy_n = lz.n;
    a.lazy_mode = lz.mode;
    a.W = rp.W;
    a.V = g.V;
    a.source = rp.source;
    a.length = rp.length;
    a.run = rp.run;
    a.seed = e.cfg.seed;
    a.thr = rp.thr;
    a.counts = rp.counts;
    a.endpoints = rp.endpoints;
    a.paths = rp.paths;
    a.out_cur = o.d_out;
    a.out_step = o.d_out + o.staging_cap;
    a.out_idx = o.d_out + 2 * o.staging_cap;
    a.out_dest = o.d_out + 3 * o.staging_cap;
    a.out_q = o.d_out + 4 * o.staging_cap;
    a.out_n = o.ctl_out_n();
    a.hist = o.ctl_hist();
    a.visits = o.ctl_visits();
    a.next = o.ctl_next();
    a.stats = o.d_stats;
    a.zc_part = kNoPart;
    a.zc_rp_base = o.zc_rp_base;
    a.rp32 = o.d_index != nullptr;
    a.zc_col_base = o.zc_col_base;
    if (o.tier_ready) {
        a.hot_on = 1;
        a.hot_words = (const uint2 *)o.d_tier;
        a.hot_off = (const uint32_t *)(o.d_tier + o.tier_off_at);
        a.hot_pool = (const uint32_t *)(o.d_tier + o.tier_pool_at);
    }
    if (o.zc_mask_any) std::memcpy(a.zc_mask, o.zc_mask, sizeof a.zc_mask);
    if (o.serve) serve_args(o, a);
    if (zero_copy) {
        a.zc_part = (uint32_t)p;
        a.zc_rp = o.zc_rp_base + (o.d_index ? 4ull : 8ull) * g.node_off[p];
        a.zc_col = o.zc_col_base + 4ull * g.edge_off[p];
    }

    const bool zc_launch = zero_copy || o.zc_mask_any;
    int grid = o.grid[rp.app];
    if (split) {
        // the cached part: its own work list and walker counter, no zero-copy set
        StepArgs c = a;
        c.n_chunk_walkers = walkers_a;
        c.work_off = o.d_work_off;
        c.n_work = (uint32_t)nw_a;
        c.next = o.ctl_next2();
        c.zc_part = kNoPart;
        std::memset(c.zc_mask, 0, sizeof c.zc_mask);
        // the zero-copy part
        a.work_chunks = o.d_work + nw_a;
        a.work_off = o.d_work_off + nw_a;
        a.n_work = (uint32_t)(nw - nw_a);
        a.n_chunk_walkers = n_chunk_walkers - walkers_a;
        a.lazy_count = 0;
        LT_CUDA_TRY(cudaEventRecord(o.ev_pre, e.s_compute));
        LT_CUDA_TRY(cudaStreamWaitEvent(o.s_aux, o.ev_pre, 0));
        Ooc::Timed tc{ev_get(o), ev_get(o), kTCompute};
        nvtxRangePushA("cached_step");
        LT_CUDA_TRY(cudaEventRecord(tc.a, o.s_aux));
        const cudaError_t lc = launch_walk_part(c, rp.app, e.sms, o.s_aux);
        nvtxRangePop();
        LT_CUDA_TRY(lc);
        LT_CUDA_TRY(cudaEventRecord(tc.b, o.s_aux));
        LT_CUDA_TRY(cudaEventRecord(o.ev_aux, o.s_aux));
        o.timed.push_back(tc);
        e.stats.computing_calls++;
        e.stats.kernel_launches++;
        e.stats.split_launches++;
        grid -= e.sms;
    }
    Ooc::Timed t{ev_get(o), ev_get(o), zc_launch ? kTZero : kTCompute};
    // NVTX ranges name the launch kind for profilers (ncu --nvtx-include)
    nvtxRangePushA(zc_launch ? "zero_copy_step" : "cached_step");
    LT_CUDA_TRY(cudaEventRecord(t.a, e.s_compute));
    const cudaError_t launched = launch_walk_part(a, rp.app, grid, e.s_compute);
    nvtxRangePop();
    LT_CUDA_TRY(launched);
    LT_CUDA_TRY(cudaEventRecord(t.b, e.s_compute));
    o.timed.push_back(t);
    if (split) LT_CUDA_TRY(cudaStreamWaitEvent(e.s_compute, o.ev_aux, 0));
    LT_CUDA_TRY(cudaEventRecord(o.ev_steps, e.s_compute));
    if (zc_launch)
        e.stats.zerocopy_calls++;
    else
        e.stats.computing_calls++;
    e.stats.kernel_launches++;
    if (deferred) {
        for (auto &d : *deferred) {
            LT_CUDA_TRY(cudaStreamWaitEvent(e.s_compute, d.second, 0));
            LT_TRY(set_entry(o, d.first, e.s_compute));
        }
        deferred->clear();
    }
    uint32_t *h_hist = (uint32_t *)o.h_ctl.ptr;
    if (dev_plan) {
        // the control block goes to the host on the copy-back stream as soon
        // as the step kernel ends; plan and bucketing follow the kernel on the
        // compute stream while the host reads it
        if (!o.ev_ctl) LT_CUDA_TRY(cudaEventCreateWithFlags(&o.ev_ctl, cudaEventDisableTiming));
        LT_CUDA_TRY(cudaStreamWaitEvent(e.s_copyback, o.ev_steps, 0));
        LT_CUDA_TRY(cudaMemcpyAsync(h_hist, o.d_ctl, 4ull * o.ctl_words, cudaMemcpyDeviceToHost, e.s_copyback));
        LT_CUDA_TRY(cudaEventRecord(o.ev_ctl, e.s_copyback));
        ScatterArgs sa{};
        sa.in_cur = a.out_cur;
        sa.in_step = a.out_step;
        sa.in_idx = a.out_idx;
        sa.in_dest = a.out_dest;
        sa.in_q = a.out_q;
        sa.n = n_in;
        sa.n_dev = o.ctl_out_n();
        sa.arena = o.d_arena;
        sa.cursor = pa.cursor;
        sa.win_off = pa.win_off;
        sa.plan_chunks = pa.plan_chunks;
        sa.P = o.P;
        sa.items = e.cfg.bucket_items;
        sa.err = o.ctl_bucket_err();
        Ooc::Timed tb{ev_get(o), ev_get(o), kTBucket};
        LT_CUDA_TRY(cudaEventRecord(tb.a, e.s_compute));
        nvtxRangePushA("bucketing");
        cudaError_t bucketed = launch_plan(pa, e.s_compute);
        if (bucketed == cudaSuccess) bucketed = launch_scatter(sa, e.device, e.s_compute);
        nvtxRangePop();
        LT_CUDA_TRY(bucketed);
        LT_CUDA_TRY(cudaEventRecord(tb.b, e.s_compute));
        o.timed.push_back(tb);
        e.stats.kernel_launches += 2;
        e.stats.device_plans++;
        e.stats.host_submit_ms += now_ms() - t_submit;
        observe_due_now(o);
        const double w0 = now_ms();
        LT_CUDA_TRY(cudaEventSynchronize(o.ev_ctl));
        e.stats.host_wait_ms += now_ms() - w0;
    } else {
        LT_CUDA_TRY(cudaMemcpyAsync(h_hist, o.d_ctl, 4ull * o.ctl_words, cudaMemcpyDeviceToHost, e.s_compute));
        e.stats.host_submit_ms += now_ms() - t_submit;
        observe_due_now(o);
        const double w0 = now_ms();
        LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
        e.stats.host_wait_ms += now_ms() - w0;
    }
    const double t_replay = now_ms();
    struct ReplayTimer {
        lt_stats &st;
        double t0;
        ~ReplayTimer() { st.host_replay_ms += now_ms() - t0; }
    } replay_timer{e.stats, t_replay};
    // an earlier bucketing pass read a tile from global memory instead of its
    // bulk copy (no walker lost, but the copy engine did not answer), or its
    // device plan did not fit (cannot happen under the bound above)
    const uint32_t bucket_err = h_hist[o.bucket_err_word()];
    if (bucket_err & 2u) return fail(LT_ERR_CAPACITY, "bucketing: the device plan ran out of free chunks");
    if (bucket_err & 1u) return fail(LT_ERR_TIMEOUT, "bucketing: a bulk copy into shared memory did not complete");
    const uint64_t staged = *(const unsigned long long *)(h_hist + o.hist_words());
    if (!dev_plan) {
        // the drained queues' chunks return to the pool
        for (uint32_t x : parts) {
            Queue &qx = o.q[x];
            for (uint32_t c : qx.dev_chunks) o.free_chunks.push_back(c);
            qx.dev_chunks.clear();
            qx.tail_fill = 0;
            refresh(o, x);
        }
    }
    if (qp) {
        qp->lazy_next += G;
        refresh(o, (uint32_t)p);
    }
    std::memcpy(o.arrivals.data(), h_hist, 4ull * o.P);
    std::memcpy(o.visits.data(), h_hist + o.P, 4ull * o.P);
    for (uint32_t x = 0; x < o.P; x++) {
        const bool cached = o.slot_of[x] >= 0;
        o.run_visits[x] += o.visits[x];
        o.run_cached_visits[x] += cached ? o.visits[x] : 0;
        o.run_cached_launches[x] += cached;
    }
    if (staged == 0) return LT_OK;

    if (dev_plan) {
        // the device planned this pass: the same arithmetic on the host
        // updates the queues' chunk lists
        plan_windows(o, h_hist, nullptr, nullptr, nullptr);
        return LT_OK;
    }
    // Plan the append of h_hist[d] walkers to each destination queue.
    uint64_t need = 0;
    for (uint32_t d = 0; d < o.P; d++) {
        if (!h_hist[d]) continue;
        const Queue &qd = o.q[d];
        const bool open_tail = !qd.dev_chunks.empty() && qd.tail_fill < kChunk;
        const uint64_t fill = open_tail ? qd.tail_fill : 0;
        need += (fill + h_hist[d] + kChunk - 1) / kChunk - (open_tail ? 1 : 0);
    }
    if (need > o.free_chunks.size()) LT_TRY(spill_until(o, need, -1));
    if (need > o.free_chunks.size()) return fail(LT_ERR_CAPACITY, "walker pool exhausted");
    uint32_t *h_cursor = (uint32_t *)o.h_plan.ptr;
    uint32_t *h_win = h_cursor + o.P;
    uint32_t *h_chunks = h_win + o.P;
    const uint64_t n_plan = plan_windows(o, h_hist, h_cursor, h_win, h_chunks);
    if (n_plan > o.plan_cap) return fail(LT_ERR_CAPACITY, "plan buffer too small");
    LT_TRY(upload(o, o.d_planbuf, o.h_plan, o.h_plan_dev, h_cursor, 2ull * o.P + n_plan));
    ScatterArgs sa{};
    sa.in_cur = a.out_cur;
    sa.in_step = a.out_step;
    sa.in_idx = a.out_idx;
    sa.in_dest = a.out_dest;
    sa.in_q = a.out_q;
    sa.n = staged;
    sa.n_dev = nullptr;
    sa.arena = o.d_arena;
    sa.cursor = o.d_planbuf;
    sa.win_off = o.d_planbuf + o.P;
    sa.plan_chunks = o.d_planbuf + 2ull * o.P;
    sa.P = o.P;
    sa.items = e.cfg.bucket_items;
    sa.err = o.ctl_bucket_err();
    Ooc::Timed tb{ev_get(o), ev_get(o), kTBucket};
    LT_CUDA_TRY(cudaEventRecord(tb.a, e.s_compute));
    nvtxRangePushA("bucketing");
    const cudaError_t bucketed = launch_scatter(sa, e.device, e.s_compute);
    nvtxRangePop();
    LT_CUDA_TRY(bucketed);
    LT_CUDA_TRY(cudaEventRecord(tb.b, e.s_compute));
    o.timed.push_back(tb);
    e.stats.kernel_launches++;
    return LT_OK;
}

// Walkers that can be created in this pass without overflowing the pool:
// after p's own chunks are released, every staged walker must fit, plus one
// partially filled tail chunk per destination.
uint64_t lazy_budget(Ooc &o, int32_t p, uint64_t left)
{
    const uint64_t own_chunks = p >= 0 ? o.q[p].dev_chunks.size() : 0;
    const uint64_t own = p >= 0 ? o.q[p].dev_count() : 0;
    const uint64_t avail = o.free_chunks.size() + own_chunks;
    if (avail <= (uint64_t)o.P + 1) return 0;
    uint64_t g = (avail - o.P - 1) * kChunk;
    g = g > own ? g - own : 0;
    if (g + own > o.staging_cap) g = o.staging_cap > own ? o.staging_cap - own : 0;
    return std::min(g, left);
}

lt_status ensure_pool(Ooc &o, uint64_t W)
{
    lt_engine &e = *o.e;
    uint64_t B = e.cfg.num_device_walkers ? e.cfg.num_device_walkers : W;
    if (B > W) B = W;
    if (B < kChunk) B = kChunk;
    const uint64_t want = (B + kChunk - 1) / kChunk + 2ull * o.P + 2;
    if (want > 0xFFFFFFF0ull) return fail(LT_ERR_CAPACITY, "walker pool too large");
    if (o.d_arena && o.n_chunks == want) return LT_OK;
    for (void *p : {(void *)o.d_arena, (void *)o.d_out, (void *)o.d_planbuf, (void *)o.d_work, (void *)o.d_work_off})
        if (p) cudaFree(p);
    host_free(o.h_plan);
    host_free(o.h_work);
    o.d_arena = nullptr;
    o.d_out = o.d_planbuf = o.d_work = nullptr;
    o.d_work_off = nullptr;
    o.n_chunks = (uint32_t)want;
    o.staging_cap = (uint64_t)o.n_chunks * kChunk;
    o.plan_cap = o.n_chunks + (uint64_t)o.P;
    o.work_cap = o.n_chunks;
    LT_TRY(dalloc(&o.d_arena, (uint64_t)o.n_chunks * kChunkBytes));
    LT_TRY(dalloc(&o.d_out, 5 * o.staging_cap));
    LT_TRY(dalloc(&o.d_planbuf, 2ull * o.P + o.plan_cap));
    LT_TRY(dalloc(&o.d_work, o.work_cap));
    LT_TRY(dalloc(&o.d_work_off, o.work_cap));
    LT_TRY(host_alloc(o.h_plan, 4 * (2ull * o.P + o.plan_cap), true));
    LT_TRY(host_alloc(o.h_work, 12 * o.work_cap + 8, true));
    host_free(o.h_planin);
    o.planin_words = 2ull * o.P + o.n_chunks;
    LT_TRY(host_alloc(o.h_planin, 2 * 4 * o.planin_words, true));
    o.h_plan_dev = o.h_work_dev = o.h_planin_dev = nullptr;
    void *dv = nullptr;
    if (o.h_planin.pinned && cudaHostGetDevicePointer(&dv, o.h_planin.ptr, 0) == cudaSuccess)
        o.h_planin_dev = (uint8_t *)dv;
    if (o.h_plan.pinned && cudaHostGetDevicePointer(&dv, o.h_plan.ptr, 0) == cudaSuccess) o.h_plan_dev = (uint8_t *)dv;
    if (o.h_work.pinned && cudaHostGetDevicePointer(&dv, o.h_work.ptr, 0) == cudaSuccess) o.h_work_dev = (uint8_t *)dv;
    cudaGetLastError();
    return LT_OK;
}

void reset_queues(Ooc &o)
{
    o.free_chunks.clear();
    for (uint32_t c = o.n_chunks; c-- > 0;) o.free_chunks.push_back(c);
    for (Queue &qq : o.q) {
        for (uint32_t h : qq.host_chunks) o.host_free.push_back(h);
        qq = Queue{};
    }
}

// graphLoadingPhase's pipeline (src/Scheduler.h:194-208): while the load of
// p is on the copy engine, drain the device queue of the cached partition the
// policy picks (getComputedPartition), one synchronous step kernel at a time,
// until the copy has finished or nothing is worth computing.  The walkers
// these kernels send to p queue there: p is published only afterwards.
lt_status overlap_load(Ooc &o, const RunParams &rp, uint32_t p, cudaEvent_t copy_done)
{
    lt_engine &e = *o.e;
    for (uint32_t k = 0; k < o.P; k++) {
        const cudaError_t q = cudaEventQuery(copy_done);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) LT_CUDA_TRY(q);
        const int32_t c = o.policy->overlap(view(o), (int32_t)p);
        if (c < 0) break;
        LT_TRY(step_and_bucket(o, rp, c, Lazy{}, false, nullptr));
        e.stats.overlap_computes++;
        drain_timers(o, false);
    }
    cudaGetLastError();
    return LT_OK;
}

// One iteration for partition p (GPUScheduler::run).
lt_status process(Ooc &o, const RunParams &rp, uint32_t p)
{
    lt_engine &e = *o.e;
    o.iteration++;
    e.stats.iterations++;
    o.last_used[p] = o.iteration;
    o.prev_computed = (int32_t)p;
    Queue &qp = o.q[p];
    SchedView v0 = view(o);
    const bool zero_copy = o.slot_of[p] < 0 && o.policy->zero_copy(v0, p, o.zc_threshold);
    if (!zero_copy) {
        e.stats.explicit_iterations++;
        std::vector<std::pair<uint32_t, cudaEvent_t>> pending;
        LT_TRY(load_partition(o, p, &pending));
        if (!pending.empty()) {
            if (e.cfg.pipeline) LT_TRY(overlap_load(o, rp, p, pending.front().second));
            for (auto &d : pending) {
                LT_CUDA_TRY(cudaStreamWaitEvent(e.s_compute, d.second, 0));
                LT_TRY(set_entry(o, d.first, e.s_compute));
            }
        }
        o.prev_loaded = (int32_t)p;
    }
    // walkerLoadingPhase: bring spilled walkers back, keeping room to make progress
    if (!qp.host_chunks.empty()) {
        const uint64_t want = qp.host_chunks.size();
        const uint64_t reserve = (uint64_t)o.P + 2;
        if (o.free_chunks.size() < want + reserve) {
            const uint64_t target = std::min<uint64_t>(want + reserve, o.n_chunks - qp.dev_chunks.size());
            lt_status s = spill_until(o, target, (int32_t)p);
            if (s != LT_OK && o.free_chunks.size() <= reserve) return s;
            clear_error();
        }
        const uint64_t room = o.free_chunks.size() > reserve ? o.free_chunks.size() - reserve : 0;
        LT_TRY(unspill(o, p, std::min<uint64_t>(want, room)));
    }
    uint64_t G = lazy_budget(o, (int32_t)p, qp.lazy_left());
    if (G == 0 && qp.lazy_left() > 0 && qp.dev_count() == 0) {
        LT_TRY(spill_until(o, (uint64_t)o.P + 2 + 1, (int32_t)p));
        G = lazy_budget(o, (int32_t)p, qp.lazy_left());
    }
    LT_TRY(step_and_bucket(o, rp, (int32_t)p, lazy_of(o, rp, (int32_t)p, qp.lazy_next, G), zero_copy, nullptr));
    drain_timers(o, false);
    SchedView v = view(o);
    o.policy->observe(v);
    return LT_OK;
}

// Walkers that can be created in a kernel that drains `chunks` chunks holding
// `walkers` walkers (the multi-partition form of lazy_budget).
uint64_t wave_lazy_budget(Ooc &o, uint64_t chunks, uint64_t walkers, uint64_t left)
{
    const uint64_t avail = o.free_chunks.size() + chunks;
    if (avail <= (uint64_t)o.P + 1) return 0;
    uint64_t g = (avail - o.P - 1) * kChunk;
    g = g > walkers ? g - walkers : 0;
    if (g + walkers > o.staging_cap) g = o.staging_cap > walkers ? o.staging_cap - walkers : 0;
    return std::min(g, left);
}

// walkers left outside the cache at or below which one kernel reads every
// uncached partition: few hops left, but each reads across the whole graph
// (past the host-memory reach of fast zero-copy reads).  c2: 2^21 walkers
// 1.06 s per run, 2^18 0.905 s, 1 (groups to the end) 0.895 s.  Serving
// keeps 2^18: at light load every step is then one sweep that finishes the
// admitted queries.
constexpr uint64_t kSweepWalkers = 1ull << 14;
constexpr uint64_t kSweepWalkersServe = 1ull << 18;
constexpr double kRefillHorizon = 512.0;          // iterations a refill is credited with at most
constexpr uint64_t kRefillHold = 128;             // iterations a partition stays before a refill may evict it
constexpr int kRefillMax = 2;                     // refill swaps started per check
constexpr uint64_t kRefillEvery = 4;              // iterations between refill checks
// zero-copy group: estimated host bytes its walkers touch.  Measured on the
// 2^33-edge graph: 128 MB 1.73 s, 256 MB 1.67 s, 512 MB 1.65 s per run (one
// kernel over every partition with tens of millions of walkers: 6.9 s)
constexpr uint64_t kZcGroupBytes = 512ull << 20;
// while serving: c4 at 1 000 queries/s, p99 220 ms with 128 MB groups and the
// reference load threshold, 525 ms with the bulk-run values
constexpr uint64_t kZcGroupBytesServe = 128ull << 20;

// Wave run.  Iteration i: publish the loads started in iteration i-1; drain,
// in one step kernel, the queues of every cached partition (the ones just
// loaded hold the walkers that queued for them) and create new walkers into
// the room the pool has; start the loads for iteration i+1 -- the partitions
// not cached with the most waiting walkers, at least the zero-copy threshold
// -- on the copy stream, so they overlap this kernel, their slots taken from
// idle cached partitions with the lowest cache_score.  When nothing is worth a
// load and no walker can be created, every partition outside the cache is
// read zero-copy in one kernel (the final phase).  Results are those of the
// reference loop: every draw is keyed by walker and step.
struct WaveState {
    explicit WaveState(uint32_t P) : score(P, 0.0), draining(P, 0), loading(P, 0) {}
    std::vector<std::pair<uint32_t, cudaEvent_t>> inflight;  // loads started, entries not yet published
    std::vector<uint32_t> parts, cand, idle;
    std::vector<double> score;  // victims' cache scores
    std::vector<char> draining, loading;
    int stalls = 0;
};

// Publish every load in flight (the compute stream waits for its copy).
lt_status publish_all(Ooc &o, WaveState &w)
{
    lt_engine &e = *o.e;
    for (auto &d : w.inflight) {
        LT_CUDA_TRY(cudaStreamWaitEvent(e.s_compute, d.second, 0));
        LT_TRY(set_entry(o, d.first, e.s_compute));
        w.loading[d.first] = 0;
    }
    w.inflight.clear();
    return LT_OK;
}

// One wave iteration (see wave_run); done = nothing waits and nothing loads.
lt_status wave_step(Ooc &o, const RunParams &rp, WaveState &w, bool &done)
{
    lt_engine &e = *o.e;
    const double t_sched = now_ms();
    const bool zc_ok = o.zc_rp_base != 0 && o.P <= kSmemPartMax && o.zc_threshold > 0;
    // A wave loads a partition once its waiting walkers would read more host
    // bytes zero-copy than the load copies.  The reference's threshold
    // (partitionSize/128/2 walkers) is that break-even at 256 bytes per
    // zero-copy hop; grouped hops cost 62 or 32 bytes, so the threshold
    // scales by 256 / bytes per hop.  Measured per run on the 2^33-edge
    // graph: host index 1x 1.63 s, 2x 1.49 s, 4x 1.47 s, 8x 1.64 s (6 300 /
    // 4 900 / 3 100 / 256 loads); resident index 4x 1.30-1.41 s, 8x
    // 1.20-1.25 s (3 100 / 256 loads).  Serving keeps the reference
    // threshold and smaller zero-copy groups: shorter steps matter more
    // there than fewer loads.
    const uint64_t load_factor = o.serve ? 1 : e.cfg.load_factor ? e.cfg.load_factor : 256 / zc_bytes_per_hop(o);
    const uint64_t load_min = !zc_ok ? 1
                              : o.zc_threshold > UINT64_MAX / load_factor ? UINT64_MAX
                                                                          : o.zc_threshold * load_factor;
    const uint64_t zc_group_bytes =
        e.cfg.zc_group_bytes ? e.cfg.zc_group_bytes : o.serve ? kZcGroupBytesServe : kZcGroupBytes;
    const uint64_t sweep_walkers =
        e.cfg.sweep_walkers ? e.cfg.sweep_walkers : o.serve ? kSweepWalkersServe : kSweepWalkers;
    const uint64_t reserve = (uint64_t)o.P + 2;
    auto &inflight = w.inflight;
    auto &parts = w.parts;
    auto &cand = w.cand;
    auto &idle = w.idle;
    auto &draining = w.draining;
    auto &loading = w.loading;
    done = false;
    {
        // publish the loads whose copies have finished; the others stay in
        // flight (not drained, not evicted) until a later iteration
        {
            size_t keep = 0;
            for (auto &d : inflight) {
                const cudaError_t q = cudaEventQuery(d.second);
                if (q == cudaSuccess) {
                    LT_TRY(set_entry(o, d.first, e.s_compute));
                    loading[d.first] = 0;
                } else {
                    if (q != cudaErrorNotReady) LT_CUDA_TRY(q);
                    cudaGetLastError();
                    inflight[keep++] = d;
                }
            }
            inflight.resize(keep);
        }
        if (o.tier_loaded && !o.tier_ready) {
            const cudaError_t q = cudaEventQuery(o.ev_tier);
            if (q == cudaSuccess)
                o.tier_ready = true;
            else if (q != cudaErrorNotReady)
                LT_CUDA_TRY(q);
            else
                cudaGetLastError();
        }
        refresh_all(o);
        bool any = false;
        for (uint32_t p = 0; p < o.P && !any; p++) any = o.waiting[p] > 0;
        if (!any) {
            LT_TRY(publish_all(o, w));
            observe_due_now(o);
            done = true;
            return LT_OK;
        }
        o.iteration++;
        e.stats.iterations++;

        // drain set: cached partitions with queued walkers; spilled ones come back first
        parts.clear();
        for (uint32_t p = 0; p < o.P; p++) {
            draining[p] = 0;
            if (o.slot_of[p] < 0 || loading[p]) continue;
            Queue &qp = o.q[p];
            if (!qp.host_chunks.empty()) {
                const uint64_t room = o.free_chunks.size() > reserve ? o.free_chunks.size() - reserve : 0;
                if (room) LT_TRY(unspill(o, p, std::min<uint64_t>(qp.host_chunks.size(), room)));
            }
            if (!qp.dev_chunks.empty()) {
                parts.push_back(p);
                draining[p] = 1;
                o.last_used[p] = o.iteration;
            }
        }

        // loads for the next kernel
        SchedView v = view(o);
        cand.clear();
        for (uint32_t p = 0; p < o.P; p++)
            if (o.slot_of[p] < 0 && o.waiting[p] >= load_min) cand.push_back(p);
        std::sort(cand.begin(), cand.end(), [&](uint32_t a, uint32_t b) {
            return o.waiting[a] != o.waiting[b] ? o.waiting[a] > o.waiting[b] : a < b;
        });
        // victims in eviction order (lowest cache score first), ordered only
        // when an eviction is considered: most iterations start no load
        bool idle_ready = false;
        auto order_idle = [&]() {
            if (idle_ready) return;
            idle_ready = true;
            idle.clear();
            for (uint32_t p = 0; p < o.P; p++)
                if (o.slot_of[p] >= 0 && !draining[p] && !loading[p] && o.waiting[p] == 0) idle.push_back(p);
            std::vector<double> &sc = w.score;
            for (uint32_t p : idle) sc[p] = o.policy->cache_score(v, p);
            std::sort(idle.begin(), idle.end(), [&](uint32_t a, uint32_t b) {
                if (sc[a] != sc[b]) return sc[a] < sc[b];
                return o.last_used[a] != o.last_used[b] ? o.last_used[a] < o.last_used[b] : a < b;
            });
        };
        size_t n_idle = 0, started = 0;
        const size_t m = std::max<size_t>(1, o.policy->wave_loads());
        for (uint32_t c : cand) {
            if (started >= m) break;
            int32_t slot = free_slot(o);
            if (slot < 0) {
                order_idle();
                if (n_idle >= idle.size()) break;
                const uint32_t w = idle[n_idle++];
                slot = o.slot_of[w];
                LT_TRY(evict_partition(o, w));
            }
            LT_TRY(start_load(o, c, slot, &inflight));
            loading[c] = 1;
            o.last_used[c] = o.iteration;
            started++;
        }
        // cold cache at a run's start: after the loads the waiting walkers
        // ask for (the source partition first), the policy's best partitions
        // go into every free slot at once; the copies overlap this and the
        // following kernels and are published as they land
        {
            std::vector<uint32_t> order;
            if (!e.cfg.no_prefill && free_slot(o) >= 0 && o.policy->prefill(v, order)) {
                for (uint32_t p : order) {
                    const int32_t slot = free_slot(o);
                    if (slot < 0) break;
                    if (o.slot_of[p] >= 0 || loading[p]) continue;
                    LT_TRY(start_load(o, p, slot, &inflight));
                    loading[p] = 1;
                    o.last_used[p] = o.iteration;
                    e.stats.prefill_loads++;
                }
            }
        }
        // Nothing worth a load but slots are free (light load, e.g. serving
        // from a cold cache): fill them with the partitions scoring highest
        // (policy score plus waiting walkers) -- no eviction, and the copies
        // overlap the kernel.
        if (cand.empty() && free_slot(o) >= 0) {
            std::vector<std::pair<double, uint32_t>> fill;
            for (uint32_t p = 0; p < o.P; p++) {
                if (o.slot_of[p] >= 0 || loading[p]) continue;
                const double sc = o.policy->cache_score(v, p) + (double)o.waiting[p];
                if (sc > 0.0) fill.push_back({sc, p});
            }
            std::sort(fill.begin(), fill.end(), [](const std::pair<double, uint32_t> &a,
                                                   const std::pair<double, uint32_t> &b) {
                return a.first != b.first ? a.first > b.first : a.second < b.second;
            });
            for (const auto &f : fill) {
                if (started >= m) break;
                const int32_t slot = free_slot(o);
                if (slot < 0) break;
                LT_TRY(start_load(o, f.second, slot, &inflight));
                loading[f.second] = 1;
                o.last_used[f.second] = o.iteration;
                started++;
            }
        }
        // Refill by forecast: with the cache full and no partition worth a
        // load by its waiting walkers, swap an idle cached partition for an
        // uncached one when the policy forecasts enough more entries for it
        // over the rest of the run: (rate_in - rate_out) x remaining
        // iterations x bytes per zero-copy hop must pay for the copy eight
        // times over, the victim must have been cached for kRefillHold
        // iterations, and at most kRefillMax swaps start per check (one
        // every kRefillEvery iterations) --
        // per-iteration forecasts are noisy: a first version (margin 2, no
        // hold, up to 8 swaps per iteration) made 3 000 swaps per c2 run and
        // doubled its host-link bytes, margin 4 with a 64-iteration hold
        // still made 550-900 without raising the cached share of entries.  Remaining iterations are
        // estimated from the walkers still to be created (at most
        // kRefillHorizon).  Policies without a forecast (batched) never
        // refill.
        if (zc_ok && cand.empty() && started < m && !o.serve && o.iteration % kRefillEvery == 0 &&
            free_slot(o) < 0 && (order_idle(), n_idle < idle.size())) {
            uint64_t left = 0;
            for (uint32_t p = 0; p < o.P; p++) left += o.lazy_left[p];
            const double made = (double)rp.W - (double)left;
            const double rest_it =
                std::min(kRefillHorizon, made > 0 ? std::max(16.0, (double)o.iteration * (double)left / made) : 16.0);
            std::vector<std::pair<double, uint32_t>> in, out;
            bool have = true;
            for (uint32_t p = 0; p < o.P && have; p++) {
                const double r = o.policy->visit_rate(v, p);
                if (r < 0) have = false;
                else if (o.slot_of[p] < 0 && !loading[p]) in.push_back({r, p});
            }
            if (have) {
                for (size_t k = n_idle; k < idle.size(); k++)
                    if (o.iteration >= o.loaded_at[idle[k]] + kRefillHold)
                        out.push_back({o.policy->visit_rate(v, idle[k]), idle[k]});
                // at most kRefillMax swaps: only the best candidates and the
                // weakest victims need ordering
                const size_t kin = std::min<size_t>(kRefillMax, in.size()), kout = std::min<size_t>(kRefillMax, out.size());
                std::partial_sort(in.begin(), in.begin() + kin, in.end(),
                                  [](const std::pair<double, uint32_t> &a, const std::pair<double, uint32_t> &b) {
                                      return a.first != b.first ? a.first > b.first : a.second < b.second;
                                  });
                std::partial_sort(out.begin(), out.begin() + kout, out.end(),
                                  [](const std::pair<double, uint32_t> &a, const std::pair<double, uint32_t> &b) {
                                      return a.first != b.first ? a.first < b.first : a.second < b.second;
                                  });
                in.resize(kin);
                out.resize(kout);
                const double hop = (double)zc_bytes_per_hop(o);
                int swaps = 0;
                for (size_t k = 0; k < in.size() && k < out.size() && started < m && swaps < kRefillMax; k++) {
                    const uint32_t pin = in[k].second, pout = out[k].second;
                    const double gain = (in[k].first - out[k].first) * rest_it * hop;
                    if (gain < 8.0 * (double)host_part_bytes(o, pin)) break;
                    swaps++;
                    const int32_t slot = o.slot_of[pout];
                    LT_TRY(evict_partition(o, pout));
                    LT_TRY(start_load(o, pin, slot, &inflight));
                    loading[pin] = 1;
                    o.last_used[pin] = o.iteration;
                    started++;
                    e.stats.refill_loads++;
                }
            }
        }
        if (started) e.stats.explicit_iterations++;
        if (!e.cfg.pipeline) {
            // no pipelining (--no-pipeline): the loads finish before this
            // iteration's kernel instead of overlapping it
            for (auto &d : inflight) {
                LT_CUDA_TRY(cudaStreamWaitEvent(e.s_compute, d.second, 0));
                LT_TRY(set_entry(o, d.first, e.s_compute));
                loading[d.first] = 0;
            }
            inflight.clear();
        }

        // walkers to create: into a readable partition if one has them
        uint64_t chunks = 0, walkers = 0;
        for (uint32_t p : parts) {
            chunks += o.q[p].dev_chunks.size();
            walkers += o.q[p].dev_count();
        }
        int32_t lazy_p = -1;
        for (int pass = 0; pass < 2 && lazy_p < 0; pass++)
            for (uint32_t p = 0; p < o.P; p++) {
                if (o.lazy_left[p] == 0 || loading[p]) continue;
                if (pass == 0 && o.slot_of[p] < 0) continue;
                if (lazy_p < 0 || o.lazy_left[p] > o.lazy_left[lazy_p]) lazy_p = (int32_t)p;
            }
        uint64_t G = lazy_p >= 0 ? wave_lazy_budget(o, chunks, walkers, o.lazy_left[lazy_p]) : 0;

        // Nothing worth a load: read partitions outside the cache zero-copy,
        // in the same kernel as the walkers created this iteration (their
        // hops through cached partitions use the issue slots that warps
        // waiting on host reads leave idle: c2 0.98 -> 0.92-0.96 s per run,
        // 1 170 -> 500 iterations, against zero-copy groups only once the
        // pool is full).  Zero-copy hops are fast only while the host lines they
        // touch stay cached, so the partitions go in groups of bounded
        // estimated footprint, most waiting walkers first; once every walker
        // exists and few are left outside the cache, one sweep makes every
        // partition readable and finishes them in a single, latency-bound
        // kernel (with walkers still to create, a sweep over the 34 GiB c2
        // graph took 75 s per run).
        std::memset(o.zc_mask, 0, sizeof o.zc_mask);
        o.zc_mask_any = false;
        bool lazy_left = false;
        for (uint32_t p = 0; p < o.P && !lazy_left; p++) lazy_left = o.lazy_left[p] > 0;
        if (zc_ok && cand.empty()) {
            uint64_t outside = 0;
            std::vector<uint32_t> group;
            for (uint32_t p = 0; p < o.P; p++)
                if (o.slot_of[p] < 0 && o.waiting[p] > 0) {
                    outside += o.waiting[p];
                    group.push_back(p);
                }
            const bool sweep = outside <= sweep_walkers && !lazy_left;
            if (!sweep) {
                // serving: the partitions whose walkers have waited longest
                // first (the latency tail of a query is its slowest walker),
                // then the most waiting walkers
                auto more = [&](uint32_t a, uint32_t b) {
                    if (o.serve && o.wait_since[a] != o.wait_since[b]) return o.wait_since[a] < o.wait_since[b];
                    return o.waiting[a] != o.waiting[b] ? o.waiting[a] > o.waiting[b] : a < b;
                };
                // host bytes a partition's walkers touch: at most the partition,
                // else about two 128-byte lines per hop (one with the index
                // resident), two hops per walker
                auto footprint = [&](uint32_t p) {
                    return std::min<uint64_t>(host_part_bytes(o, p), (o.d_index ? 256 : 512) * o.waiting[p]);
                };
                // most waiting walkers first; a group holds few partitions,
                // so only a prefix is ordered (64 at a time)
                uint64_t bytes = 0;
                size_t n = 0, sorted = 0;
                while (n < group.size()) {
                    if (n == sorted) {
                        const size_t k = std::min<size_t>(group.size(), sorted + 64);
                        std::partial_sort(group.begin() + sorted, group.begin() + k, group.end(), more);
                        sorted = k;
                    }
                    if (n > 0 && bytes + footprint(group[n]) > zc_group_bytes) break;
                    bytes += footprint(group[n++]);
                }
                group.resize(n);
            } else {
                group.clear();
                for (uint32_t p = 0; p < o.P; p++)
                    if (o.slot_of[p] < 0) group.push_back(p);
            }
            if (!group.empty()) {
                if (sweep)
                    e.stats.zerocopy_sweeps++;
                else
                    e.stats.zerocopy_groups++;
            }
            for (uint32_t p : group) {
                o.zc_mask[p >> 5] |= 1u << (p & 31);
                o.zc_mask_any = true;
                Queue &qp = o.q[p];
                if (!qp.host_chunks.empty()) {
                    const uint64_t room = o.free_chunks.size() > reserve ? o.free_chunks.size() - reserve : 0;
                    if (room) LT_TRY(unspill(o, p, std::min<uint64_t>(qp.host_chunks.size(), room)));
                }
                if (!qp.dev_chunks.empty()) {
                    parts.push_back(p);
                    chunks += qp.dev_chunks.size();
                    walkers += qp.dev_count();
                }
            }
            if (lazy_p >= 0) G = wave_lazy_budget(o, chunks, walkers, o.lazy_left[lazy_p]);
        }
        if (parts.empty() && G == 0 && started == 0 && !inflight.empty()) {
            // nothing to compute until a load lands: wait for the oldest one
            // (copies finish in the order they were issued on the copy stream)
            o.zc_mask_any = false;
            LT_CUDA_TRY(cudaEventSynchronize(inflight.front().second));
            LT_TRY(set_entry(o, inflight.front().first, e.s_compute));
            loading[inflight.front().first] = 0;
            inflight.erase(inflight.begin());
            return LT_OK;
        }
        if (parts.empty() && G == 0 && started == 0) {
            // Nothing readable holds walkers, none can be created and nothing
            // is loading: the pool is full of walkers queued outside the cache
            // while the cached partitions wait for spilled or uncreated ones.
            // Spill to make room, then try again.
            o.zc_mask_any = false;
            if (++w.stalls > 2)
                return fail(LT_ERR_CAPACITY, "wave scheduler cannot make progress (walker pool or cache too small)");
            LT_TRY(spill_until(o, std::min<uint64_t>(o.n_chunks, reserve + 64), -1));
            return LT_OK;
        }
        w.stalls = 0;
        const Lazy lz = lazy_p >= 0 ? lazy_of(o, rp, lazy_p, o.q[lazy_p].lazy_next, G) : Lazy{};
        e.stats.host_sched_ms += now_ms() - t_sched;
        LT_TRY(step_and_bucket_parts(o, rp, parts, lazy_p, lz, false, nullptr));
        o.zc_mask_any = false;
        o.observe_due = true;
    }
    return LT_OK;
}

lt_status ckpt_point(Ooc &o, const RunParams &rp, bool &stop);

lt_status wave_run(Ooc &o, const RunParams &rp, bool &stop)
{
    WaveState w(o.P);
    bool done = false;
    stop = false;
    while (!done) {
        LT_TRY(wave_step(o, rp, w, done));
        if (done) break;
        LT_TRY(ckpt_point(o, rp, stop));
        if (stop) {
            observe_due_now(o);
            // leave the cache consistent: loads in flight land and are published
            lt_engine &e = *o.e;
            for (auto &d : w.inflight) {
                LT_CUDA_TRY(cudaStreamWaitEvent(e.s_compute, d.second, 0));
                LT_TRY(set_entry(o, d.first, e.s_compute));
            }
            LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
            return LT_OK;
        }
    }
    return LT_OK;
}

}  // namespace

lt_status ooc_create(lt_engine *e, Ooc **out)
{
    Ooc *o = new Ooc();
    o->e = e;
    o->g = e->g;
    lt_graph &g = *e->g;
    o->P = g.P();
    o->K = std::min<uint32_t>(e->cfg.num_device_partitions, o->P);
    if (o->K < 1) o->K = 1;
    o->ctl_words = o->hist_words() + 8;
    auto bail = [&](lt_status s) {
        ooc_destroy(o);
        return s;
    };
    // The vertex index goes to the device first, compact: 4 (V+1) bytes
    // (1.46 GB at 2^30 vertices), each vertex's first edge as a u32 offset
    // from its partition's first edge (a partition's edges fit 32 bits); the
    // partition's edge count ends its last row.  Where it does not fit, the
    // slots carry rowptr slices.
    if (e->cfg.resident_index && g.max_edges < (1ull << 32)) {
        std::vector<uint32_t> idx((uint64_t)g.V + 1, 0);
        const uint64_t *rp = g.rowptr();
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t p = 0; p < (int64_t)o->P; p++)
            for (uint64_t v = g.node_off[p]; v < g.node_off[p + 1]; v++) idx[v] = (uint32_t)(rp[v] - g.edge_off[p]);
        if (dalloc(&o->d_index, (uint64_t)g.V + 1) != LT_OK ||
            cudaMemcpy(o->d_index, idx.data(), 4ull * ((uint64_t)g.V + 1), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            clear_error();
            if (o->d_index) cudaFree(o->d_index);
            o->d_index = nullptr;
        }
    }
    uint64_t max_slot = 0;
    for (uint32_t p = 0; p < o->P; p++) max_slot = std::max<uint64_t>(max_slot, host_part_bytes(*o, p) + 16);
    o->slot_stride = (max_slot + 255) & ~255ull;
    // -p P gives the graph P x partitionSize bytes of device memory, as the
    // reference allocates (src/GraphLoader.h:175-178); a resident vertex
    // index is paid from that budget, leaving fewer slots.  Where it leaves
    // none, the slots carry rowptr slices instead.
    if (o->d_index) {
        const uint64_t budget = (uint64_t)o->K * g.part_bytes, index_bytes = 4ull * ((uint64_t)g.V + 1);
        uint64_t fit = budget > index_bytes ? (budget - index_bytes) / o->slot_stride : 0;
        // the hot-vertex tier takes its share of what the index leaves
        const bool wave = e->cfg.sched == LT_SCHED_LEARNED || e->cfg.sched == LT_SCHED_FREQUENCY ||
                          e->cfg.sched == LT_SCHED_BATCHED;
        if (e->cfg.hot_tier > 0 && wave && fit >= 2 && g.max_edges < (1ull << 31) && o->P <= kSmemPartMax) {
            const uint64_t avail = budget - index_bytes;
            const uint64_t want = (avail / 100 * std::min<uint64_t>((uint64_t)e->cfg.hot_tier, 90)) & ~255ull;
            o->tier_words = ((uint64_t)g.V + 31) / 32;
            const uint64_t left = (avail - want) / o->slot_stride;
            if (want > 8 * o->tier_words + 4096 && left >= 1) {
                o->tier_bytes = want;
                fit = left;
            }
        }
        if (fit >= 1) {
            o->K = (uint32_t)std::min<uint64_t>(o->K, fit);
        } else {
            cudaFree(o->d_index);
            o->d_index = nullptr;
            max_slot = 0;
            for (uint32_t p = 0; p < o->P; p++) max_slot = std::max<uint64_t>(max_slot, host_part_bytes(*o, p) + 16);
        }
    }
    if (!o->d_index) o->slot_stride = std::max<uint64_t>((max_slot + 255) & ~255ull, (g.part_bytes + 16 + 255) & ~255ull);
    lt_status s = dalloc(&o->d_slots, (uint64_t)o->K * o->slot_stride);
    if (s == LT_OK) s = dalloc(&o->d_node_off, o->P + 1);
    if (s == LT_OK) s = dalloc(&o->d_edge_off, o->P + 1);
    if (s == LT_OK) s = dalloc(&o->d_rp, o->P);
    if (s == LT_OK) s = dalloc(&o->d_col, o->P);
    if (s == LT_OK) s = dalloc(&o->d_ctl, o->ctl_words);
    if (s == LT_OK) s = dalloc(&o->d_stats, 8);
    if (s == LT_OK) s = host_alloc(o->h_ctl, 4 * o->ctl_words, true);
    if (s == LT_OK && (cudaStreamCreateWithFlags(&o->s_aux, cudaStreamNonBlocking) != cudaSuccess ||
                       cudaEventCreateWithFlags(&o->ev_steps, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&o->ev_pre, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&o->ev_aux, cudaEventDisableTiming) != cudaSuccess))
        s = fail(LT_ERR_CUDA, "stream / event creation failed");
    if (s == LT_OK && o->tier_bytes) {
        s = dalloc(&o->d_tier, o->tier_bytes);
        if (s == LT_OK) s = host_alloc(o->h_tier, o->tier_bytes, true);
        if (s == LT_OK && cudaEventCreateWithFlags(&o->ev_tier, cudaEventDisableTiming) != cudaSuccess)
            s = fail(LT_ERR_CUDA, "event creation failed");
    }
    if (s != LT_OK) return bail(s);
    if (cudaMemcpy(o->d_node_off, g.node_off.data(), 4ull * (o->P + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(o->d_edge_off, g.edge_off.data(), 8ull * (o->P + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(o->d_rp, 0, 8ull * o->P) != cudaSuccess || cudaMemset(o->d_col, 0, 8ull * o->P) != cudaSuccess ||
        cudaMemset(o->d_ctl, 0, 4ull * o->ctl_words) != cudaSuccess)
        return bail(fail(LT_ERR_CUDA, "partition table upload failed"));
    o->slot_of.assign(o->P, -1);
    o->part_in_slot.assign(o->K, -1);
    o->last_used.assign(o->P, 0);
    o->loaded_at.assign(o->P, 0);
    o->h_rp.assign(o->P, 0);
    o->h_col.assign(o->P, 0);
    o->arrivals.assign(o->P, 0);
    o->visits.assign(o->P, 0);
    o->waiting.assign(o->P, 0);
    o->wait_since.assign(o->P, 0);
    o->lazy_left.assign(o->P, 0);
    o->dev_waiting.assign(o->P, 0);
    o->run_visits.assign(o->P, 0);
    o->run_cached_visits.assign(o->P, 0);
    o->run_cached_launches.assign(o->P, 0);
    o->q.assign(o->P, Queue{});
    if (e->cfg.sched == LT_SCHED_FIFO) {
        o->policy.reset(new FifoPolicy());
    } else if (e->cfg.sched == LT_SCHED_BATCHED) {
        o->policy.reset(new BatchedPolicy());
    } else if (e->cfg.sched == LT_SCHED_LEARNED || e->cfg.sched == LT_SCHED_FREQUENCY) {
        Policy *lp = nullptr;
        s = make_learned_policy(g, e->device, e->cfg.sched == LT_SCHED_LEARNED, &lp);
        if (s != LT_OK) return bail(s);
        o->policy.reset(lp);
    } else {
        o->policy.reset(new Policy());
    }
    o->zc_threshold = e->cfg.zerocopy_threshold == UINT64_MAX ? g.part_bytes / 128 / 2 : e->cfg.zerocopy_threshold;
    if (g.rowptr_buf.pinned && g.col_buf.pinned) {
        void *rp_dev = nullptr, *col_dev = nullptr;
        if (cudaHostGetDevicePointer(&rp_dev, (void *)g.rowptr(), 0) != cudaSuccess ||
            cudaHostGetDevicePointer(&col_dev, (void *)g.col(), 0) != cudaSuccess)
            return bail(fail(LT_ERR_CUDA, "pinned graph is not mapped for zero-copy reads"));
        o->zc_rp_base = (unsigned long long)(uintptr_t)(o->d_index ? (void *)o->d_index : rp_dev);
        o->zc_col_base = (unsigned long long)(uintptr_t)col_dev;
    } else {
        o->zc_threshold = 0;  // the graph is not in pinned memory: always load
        o->tier_bytes = 0;    // (the tier's kernel path reads the index through zc_rp_base)
    }
    const size_t smem = part_smem(o->P);
    if (smem > 64 * 1024) return bail(fail(LT_ERR_UNSUPPORTED, "partition count %u needs %zu bytes of shared memory", o->P, smem));
    for (int app = 0; app < 3; app++) o->grid[app] = part_grid(app, 0, e->device, smem, e->cfg.ctas_per_sm);
    *out = o;
    return LT_OK;
}

void ooc_destroy(Ooc *o)
{
    if (!o) return;
    drain_timers(*o, true);
    for (void *p : {(void *)o->d_index, (void *)o->d_slots, (void *)o->d_node_off, (void *)o->d_edge_off, (void *)o->d_rp, (void *)o->d_col,
                    (void *)o->d_arena, (void *)o->d_out, (void *)o->d_ctl, (void *)o->d_planbuf, (void *)o->d_work,
                    (void *)o->d_work_off, (void *)o->d_stats})
        if (p) cudaFree(p);
    for (HostBuf &b : o->host_slabs) host_free(b);
    host_free(o->h_ctl);
    host_free(o->h_plan);
    host_free(o->h_work);
    host_free(o->h_planin);
    host_free(o->h_tier);
    if (o->d_tier) cudaFree(o->d_tier);
    if (o->ev_tier) cudaEventDestroy(o->ev_tier);
    if (o->ev_ctl) cudaEventDestroy(o->ev_ctl);
    for (cudaEvent_t ev : {o->ev_steps, o->ev_pre, o->ev_aux})
        if (ev) cudaEventDestroy(ev);
    if (o->s_aux) cudaStreamDestroy(o->s_aux);
    for (cudaEvent_t ev : o->ev_free) cudaEventDestroy(ev);
    delete o;
}

void ooc_policy_stats(const Ooc *o, lt_policy_stats &s) { o->policy->stats(s); }

// Autotuner of the out-of-core engine.  It times cold-cache PPR trial runs
// (from the vertex with the most out-edges, as many walkers as the device
// pool holds, at most 2^26; the best of three per setting) and walks the
// runtime knobs one at a time, keeping each value that shortens the trial by
// 5 % or more (coordinate descent; with a 3 % margin it once kept 256 MiB
// zero-copy groups that were 3.4 % faster on the trial and 5 % slower on the
// c2 run): the
// zero-copy group footprint and the load threshold factor of wave runs, the
// step kernel's resident CTAs per SM and the bucketing tile.  Every knob
// changes only the schedule, so results are unchanged.  The walker chunk
// (8192 walkers) is not tuned: it is the unit of the host spill slabs and of
// the checkpoint file.
lt_status ooc_autotune(lt_engine *e, lt_ooc_tune *out)
{
    Ooc &o = *e->ooc;
    lt_graph &g = *e->g;
    if (o.serve) return fail(LT_ERR_INVALID, "the engine is serving");
    uint32_t src = 0;
    for (uint32_t v = 0; v < g.V; v++)
        if (g.rowptr()[v + 1] - g.rowptr()[v] > g.rowptr()[src + 1] - g.rowptr()[src]) src = v;
    const uint64_t pool = e->cfg.num_device_walkers ? e->cfg.num_device_walkers : (1ull << 26);
    const uint64_t W = std::max<uint64_t>(1, std::min<uint64_t>(std::min<uint64_t>(pool, 1ull << 26), 2ull * g.V));
    const int occ = part_grid(kPPR, 0, e->device, part_smem(o.P), 0) / std::max(1, e->sms);
    const lt_engine_cfg keep = e->cfg;
    auto trial = [&](double &ms) -> lt_status {
        for (int app = 0; app < 3; app++) o.grid[app] = part_grid(app, 0, e->device, part_smem(o.P), e->cfg.ctas_per_sm);
        ms = 1e30;
        for (int rep = 0; rep < 3; rep++) {
            LT_TRY(ooc_drop_cache(&o));
            LT_TRY(ooc_run(e, kPPR, kStartSource, src, W, 0, 1, 0, 0.15f, nullptr, nullptr, nullptr));
            ms = std::min(ms, e->stats.running_ms);
        }
        return LT_OK;
    };
    double best = 0;
    lt_status st = trial(best);
    const double first = best;
    struct Knob {
        uint64_t *u64;
        uint32_t *u32;
        int *i32;
        std::vector<uint64_t> values;
    };
    std::vector<Knob> knobs;
    knobs.push_back({&e->cfg.zc_group_bytes, nullptr, nullptr, {256ull << 20, 512ull << 20, 1024ull << 20}});
    knobs.push_back({nullptr, &e->cfg.load_factor, nullptr, {4, 8, 16}});
    std::vector<uint64_t> ctas;
    for (int c = occ; c >= 1 && c >= occ - 2; c--) ctas.push_back((uint64_t)c);
    knobs.push_back({nullptr, nullptr, &e->cfg.ctas_per_sm, ctas});
    knobs.push_back({nullptr, nullptr, &e->cfg.bucket_items, {16, 8}});
    for (const Knob &k : knobs) {
        if (st != LT_OK) break;
        const uint64_t was = k.u64 ? *k.u64 : k.u32 ? *k.u32 : (uint64_t)*k.i32;
        uint64_t pick = was;
        for (uint64_t val : k.values) {
            if (k.u64) *k.u64 = val;
            if (k.u32) *k.u32 = (uint32_t)val;
            if (k.i32) *k.i32 = (int)val;
            double ms = 0;
            st = trial(ms);
            if (st != LT_OK) break;
            if (ms < best * 0.95) {
                best = ms;
                pick = val;
            }
        }
        if (k.u64) *k.u64 = pick;
        if (k.u32) *k.u32 = (uint32_t)pick;
        if (k.i32) *k.i32 = (int)pick;
    }
    if (st != LT_OK) {
        e->cfg = keep;
        for (int app = 0; app < 3; app++) o.grid[app] = part_grid(app, 0, e->device, part_smem(o.P), e->cfg.ctas_per_sm);
        return st;
    }
    for (int app = 0; app < 3; app++) o.grid[app] = part_grid(app, 0, e->device, part_smem(o.P), e->cfg.ctas_per_sm);
    LT_TRY(ooc_drop_cache(&o));
    out->tuned = 1;
    out->trial_walkers = W;
    out->zc_group_bytes = e->cfg.zc_group_bytes;
    out->load_factor = e->cfg.load_factor;
    out->ctas_per_sm = e->cfg.ctas_per_sm;
    out->bucket_items = e->cfg.bucket_items;
    out->default_ms = first;
    out->tuned_ms = best;
    return LT_OK;
}

void ooc_partition_stats(const Ooc *o, uint64_t *visits, uint64_t *cached_visits, uint64_t *cached_launches)
{
    for (uint32_t p = 0; p < o->P; p++) {
        if (visits) visits[p] = o->run_visits[p];
        if (cached_visits) cached_visits[p] = o->run_cached_visits[p];
        if (cached_launches) cached_launches[p] = o->run_cached_launches[p];
    }
}

lt_status ooc_drop_cache(Ooc *o)
{
    lt_engine &e = *o->e;
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_copy));
    LT_TRY(tier_unload(*o));
    for (uint32_t p = 0; p < o->P; p++)
        if (o->slot_of[p] >= 0) LT_TRY(evict_partition(*o, p));
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    o->policy->reset();
    return LT_OK;
}

// ------------------------------------------------------------- checkpoints
//
// A checkpoint is the state of a run between two scheduler iterations: every
// walker is then in a partition queue (device or host chunks) or not yet
// created, so the file holds (little-endian)
//   "LTCKPT01" | u32 version | u32 app, start, source, length, runs, run_base,
//   run_index, flags (1 counts, 2 endpoints, 4 paths) | u64 W | f32 prob |
//   u64 seed | u32 V | u64 E | u32 P | u64 partition-table hash |
//   u64 iteration | u64 device stats[8] |
//   counts u64[V] | endpoints u32[W] | paths u32[W (length+1)] |
//   per partition: u64 lazy_total, lazy_next, n | u32 cur[n], step[n],
//   idx[n], query[n].
// The cache is not saved: a resumed run starts from a cold cache, and since
// every draw is keyed by walker and step its results equal those of the run
// that was never interrupted.  A file is trusted no further than it can be
// checked: the header must describe a run the engine could have started
// (source inside the graph, probability and length in range, the output
// flags of the app), the partition table must hash to the engine's, each
// partition's creation progress must be the one its start mode gives, and
// every queued walker must lie in its partition, with an index below W and
// a step the app can reach -- a corrupt record would otherwise become an
// out-of-range device access in the step kernel.
namespace {

constexpr char kCkptMagic[8] = {'L', 'T', 'C', 'K', 'P', 'T', '0', '1'};
constexpr uint32_t kCkptVersion = 2;

struct CkptHeader {
    uint32_t app = 0, start = 0, source = 0, length = 0, runs = 1, run_base = 0, run_index = 0, flags = 0;
    uint64_t W = 0;
    float prob = 0.f;
    uint64_t seed = 0;
    uint32_t V = 0;
    uint64_t E = 0;
    uint32_t P = 0;
    uint64_t part_hash = 0;
    uint64_t iteration = 0;
};

// FNV-1a over the partition table (partition size, node and edge offsets):
// a checkpoint resumes only on an engine whose partitions have the same
// boundaries, since its per-partition creation progress refers to them.
uint64_t part_table_hash(const lt_graph &g)
{
    uint64_t h = 0xcbf29ce484222325ull;
    auto mix = [&](const void *p, size_t n) {
        const uint8_t *b = static_cast<const uint8_t *>(p);
        for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 0x100000001b3ull;
    };
    mix(&g.part_bytes, sizeof g.part_bytes);
    mix(g.node_off.data(), 4 * g.node_off.size());
    mix(g.edge_off.data(), 8 * g.edge_off.size());
    return h;
}

struct Writer {
    FILE *f;
    bool ok = true;
    void put(const void *p, size_t n) { ok = ok && (n == 0 || fwrite(p, 1, n, f) == n); }
    void u32(uint32_t v) { put(&v, 4); }
    void u64(uint64_t v) { put(&v, 8); }
};

struct Reader {
    FILE *f;
    bool ok = true;
    void get(void *p, size_t n) { ok = ok && (n == 0 || fread(p, 1, n, f) == n); }
    uint32_t u32()
    {
        uint32_t v = 0;
        get(&v, 4);
        return v;
    }
    uint64_t u64()
    {
        uint64_t v = 0;
        get(&v, 8);
        return v;
    }
};

void put_header(Writer &w, const CkptHeader &h)
{
    w.put(kCkptMagic, 8);
    w.u32(kCkptVersion);
    for (uint32_t v : {h.app, h.start, h.source, h.length, h.runs, h.run_base, h.run_index, h.flags}) w.u32(v);
    w.u64(h.W);
    w.put(&h.prob, 4);
    w.u64(h.seed);
    w.u32(h.V);
    w.u64(h.E);
    w.u32(h.P);
    w.u64(h.part_hash);
    w.u64(h.iteration);
}

lt_status get_header(Reader &r, const char *path, CkptHeader &h)
{
    char magic[8];
    r.get(magic, 8);
    const uint32_t version = r.u32();
    if (!r.ok || std::memcmp(magic, kCkptMagic, 8) != 0) return fail(LT_ERR_FORMAT, "%s: not a checkpoint", path);
    if (version != kCkptVersion) return fail(LT_ERR_FORMAT, "%s: checkpoint version %u", path, version);
    uint32_t *f32[] = {&h.app, &h.start, &h.source, &h.length, &h.runs, &h.run_base, &h.run_index, &h.flags};
    for (uint32_t *p : f32) *p = r.u32();
    h.W = r.u64();
    r.get(&h.prob, 4);
    h.seed = r.u64();
    h.V = r.u32();
    h.E = r.u64();
    h.P = r.u32();
    h.part_hash = r.u64();
    h.iteration = r.u64();
    if (!r.ok) return fail(LT_ERR_FORMAT, "%s: truncated checkpoint header", path);
    if (h.app > kWalk || h.start > kStartPerVertex || h.run_index >= h.runs || h.W >= (1ull << 32) || h.W == 0 ||
        h.V == 0 || h.P == 0 || h.P > h.V)
        return fail(LT_ERR_FORMAT, "%s: inconsistent checkpoint header", path);
    // the checks run_setup and the engine entry points make on a fresh run
    if (h.start == kStartSource && h.source >= h.V)
        return fail(LT_ERR_FORMAT, "%s: source %u outside the graph's %u vertices", path, h.source, h.V);
    if (h.app == kPPR && !(h.prob > 0.0f && h.prob <= 1.0f))
        return fail(LT_ERR_FORMAT, "%s: PPR stop probability outside (0, 1]", path);
    if (h.app == kPageRank && !(h.prob >= 0.0f && h.prob <= 1.0f))
        return fail(LT_ERR_FORMAT, "%s: PageRank probability outside [0, 1]", path);
    if (h.app != kPPR && h.length == 0) return fail(LT_ERR_FORMAT, "%s: walk length 0", path);
    const uint32_t want_flags = h.app == kWalk ? (h.flags & 6u) : 1u;  // counts, or endpoints / paths
    if (h.flags != want_flags)
        return fail(LT_ERR_FORMAT, "%s: output flags %u do not match the app", path, h.flags);
    return LT_OK;
}

lt_status write_checkpoint(Ooc &o, const RunParams &rp)
{
    lt_engine &e = *o.e;
    lt_graph &g = *o.g;
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_copyback));
    CkptHeader h;
    h.app = rp.app;
    h.start = rp.start;
    h.source = rp.source;
    h.length = rp.length;
    h.runs = o.run_runs;
    h.run_base = o.run_base;
    h.run_index = o.run_index;
    h.flags = (rp.counts ? 1u : 0u) | (rp.endpoints ? 2u : 0u) | (rp.paths ? 4u : 0u);
    h.W = rp.W;
    h.prob = o.run_prob;
    h.seed = e.cfg.seed;
    h.V = g.V;
    h.E = g.E;
    h.P = o.P;
    h.part_hash = part_table_hash(g);
    h.iteration = o.iteration;
    const std::string tmp = o.ckpt_path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return fail(LT_ERR_IO, "cannot write checkpoint %s", tmp.c_str());
    Writer w{f};
    put_header(w, h);
    unsigned long long hs[8];
    cudaError_t ce = cudaMemcpy(hs, o.d_stats, sizeof hs, cudaMemcpyDeviceToHost);
    w.put(hs, sizeof hs);
    if (ce == cudaSuccess && rp.counts) {
        std::vector<uint64_t> c(g.V);
        ce = cudaMemcpy(c.data(), rp.counts, 8ull * g.V, cudaMemcpyDeviceToHost);
        w.put(c.data(), 8ull * g.V);
    }
    if (ce == cudaSuccess && rp.endpoints) {
        std::vector<uint32_t> v(rp.W);
        ce = cudaMemcpy(v.data(), rp.endpoints, 4ull * rp.W, cudaMemcpyDeviceToHost);
        w.put(v.data(), 4ull * rp.W);
    }
    if (ce == cudaSuccess && rp.paths) {
        const uint64_t n = rp.W * ((uint64_t)rp.length + 1);
        std::vector<uint32_t> v(n);
        ce = cudaMemcpy(v.data(), rp.paths, 4ull * n, cudaMemcpyDeviceToHost);
        w.put(v.data(), 4ull * n);
    }
    std::vector<uint32_t> chunk(4ull * kChunk), fld[4];
    for (uint32_t p = 0; p < o.P && ce == cudaSuccess && w.ok; p++) {
        const Queue &q = o.q[p];
        for (auto &v : fld) v.clear();
        auto take = [&](const uint32_t *c, uint32_t m) {
            for (int k = 0; k < 4; k++) fld[k].insert(fld[k].end(), c + (uint64_t)k * kChunk, c + (uint64_t)k * kChunk + m);
        };
        for (size_t c = 0; c < q.dev_chunks.size() && ce == cudaSuccess; c++) {
            ce = cudaMemcpy(chunk.data(), o.d_arena + (uint64_t)q.dev_chunks[c] * kChunkBytes, kChunkBytes,
                            cudaMemcpyDeviceToHost);
            take(chunk.data(), c + 1 == q.dev_chunks.size() ? q.tail_fill : kChunk);
        }
        for (uint32_t hc : q.host_chunks) take(reinterpret_cast<const uint32_t *>(o.host_chunk(hc)), kChunk);
        w.u64(q.lazy_total);
        w.u64(q.lazy_next);
        w.u64(fld[0].size());
        for (auto &v : fld) w.put(v.data(), 4ull * v.size());
    }
    const bool ok = w.ok && std::fclose(f) == 0 && ce == cudaSuccess;
    if (!ok) {
        std::remove(tmp.c_str());
        if (ce != cudaSuccess) return fail(LT_ERR_CUDA, "checkpoint copy: %s", cudaGetErrorString(ce));
        return fail(LT_ERR_IO, "short write of checkpoint %s", tmp.c_str());
    }
    if (std::rename(tmp.c_str(), o.ckpt_path.c_str()) != 0)
        return fail(LT_ERR_IO, "cannot move checkpoint into %s", o.ckpt_path.c_str());
    return LT_OK;
}

// Walkers partition p creates lazily in a fresh run of the checkpoint's
// start mode (run_prepare): all W at the source's partition, per-vertex
// starts spread by vertex range, none for uniform starts.
uint64_t expected_lazy(const Ooc &o, const CkptHeader &h, uint32_t p)
{
    const lt_graph &g = *o.g;
    if (h.start == kStartSource) return g.find_partition(h.source) == p ? h.W : 0;
    if (h.start == kStartPerVertex) {
        const uint64_t wraps = h.W / g.V, rem = h.W % g.V;
        const uint64_t nb = g.node_off[p], n = g.node_off[p + 1] - nb;
        const uint64_t tail = rem > nb ? std::min<uint64_t>(rem - nb, n) : 0;
        return wraps * n + tail;
    }
    return 0;
}

// Rebuild the queues of a checkpoint: full chunks on the device while room
// is left (else spilled to host), each partition's partial chunk last on the
// device.  Every record is checked before anything is uploaded.
lt_status read_queues(Ooc &o, Reader &r, const char *path, const CkptHeader &h)
{
    const uint64_t reserve = (uint64_t)o.P + 2;
    HostBuf stage;
    LT_TRY(host_alloc(stage, kChunkBytes, true));
    uint32_t *sc = static_cast<uint32_t *>(stage.ptr);
    std::vector<uint32_t> fld[4];
    lt_status st = LT_OK;
    for (uint32_t p = 0; p < o.P && st == LT_OK; p++) {
        Queue &q = o.q[p];
        q.lazy_total = r.u64();
        q.lazy_next = r.u64();
        const uint64_t n = r.u64();
        if (!r.ok || q.lazy_next > q.lazy_total || q.lazy_total != expected_lazy(o, h, p) || n > h.W) {
            st = fail(LT_ERR_FORMAT, "%s: truncated or inconsistent queue of partition %u", path, p);
            break;
        }
        for (auto &v : fld) {
            v.resize(n);
            r.get(v.data(), 4ull * n);
        }
        if (!r.ok) {
            st = fail(LT_ERR_FORMAT, "%s: truncated queue of partition %u", path, p);
            break;
        }
        const uint32_t nb = o.g->node_off[p], ne = o.g->node_off[p + 1];
        for (uint64_t i = 0; i < n; i++) {
            const uint32_t cur = fld[0][i], step = fld[1][i], idx = fld[2][i], qs = fld[3][i];
            // a queued walker still needs the graph: PPR step >= 2, PageRank /
            // generic walk 1 <= step <= length
            const bool step_ok = h.app == kPPR ? step >= 2 : step >= 1 && step <= h.length;
            if (cur < nb || cur >= ne || idx >= h.W || qs != 0 || !step_ok) {
                st = fail(LT_ERR_FORMAT, "%s: walker %llu of partition %u is invalid (vertex %u, step %u, index %u)",
                          path, (unsigned long long)i, p, cur, step, idx);
                break;
            }
        }
        if (st != LT_OK) break;
        for (uint64_t b = 0; b < n && st == LT_OK; b += kChunk) {
            const uint32_t m = (uint32_t)std::min<uint64_t>(kChunk, n - b);
            const bool last = b + m == n;
            if (m == kChunk && !last && o.free_chunks.size() <= reserve + 1) {
                uint32_t hid;
                st = host_chunk_alloc(o, hid);
                if (st != LT_OK) break;
                uint32_t *hc = reinterpret_cast<uint32_t *>(o.host_chunk(hid));
                for (int k = 0; k < 4; k++) std::memcpy(hc + (uint64_t)k * kChunk, fld[k].data() + b, 4ull * kChunk);
                q.host_chunks.push_back(hid);
                continue;
            }
            if (o.free_chunks.empty()) {
                st = fail(LT_ERR_CAPACITY, "walker pool too small for the checkpoint's queues");
                break;
            }
            for (int k = 0; k < 4; k++) std::memcpy(sc + (uint64_t)k * kChunk, fld[k].data() + b, 4ull * m);
            const uint32_t c = o.free_chunks.back();
            o.free_chunks.pop_back();
            if (cudaMemcpy(o.d_arena + (uint64_t)c * kChunkBytes, sc, kChunkBytes, cudaMemcpyHostToDevice) != cudaSuccess) {
                cudaGetLastError();
                st = fail(LT_ERR_CUDA, "checkpoint upload failed");
                break;
            }
            q.dev_chunks.push_back(c);
            q.tail_fill = m;
        }
        refresh(o, p);
    }
    host_free(stage);
    return st;
}

}  // namespace

namespace {

lt_status ckpt_point(Ooc &o, const RunParams &rp, bool &stop)
{
    stop = false;
    if (o.ckpt_every == 0 || o.ckpt_path.empty() || o.iteration % o.ckpt_every != 0) return LT_OK;
    LT_TRY(write_checkpoint(o, rp));
    stop = o.ckpt_stop;
    return LT_OK;
}

// Queues of a fresh run: the start mode's walkers, not yet created (source,
// per-vertex) or created and bucketed right away (uniform starts,
// createWalkers).
lt_status run_prepare(Ooc &o, const RunParams &rp)
{
    lt_graph &g = *o.g;
    o.policy->run_start();
    // the tier holds graph data: any walk may read it, whichever built it
    if (o.tier_built && !o.serve) LT_TRY(tier_load(o));
    o.e->stats.hot_vertices = o.tier_loaded ? o.tier_hot : 0;
    reset_queues(o);
    refresh_all(o);
    o.prev_computed = -1;
    if (rp.start == kStartSource) {
        o.q[g.find_partition(rp.source)].lazy_total = rp.W;
    } else if (rp.start == kStartPerVertex) {
        const uint64_t wraps = rp.W / g.V, rem = rp.W % g.V;
        for (uint32_t p = 0; p < o.P; p++) {
            const uint64_t nb = g.node_off[p], n = g.node_off[p + 1] - nb;
            const uint64_t tail = rem > nb ? std::min<uint64_t>(rem - nb, n) : 0;
            o.q[p].lazy_total = wraps * n + tail;
        }
    } else {
        uint64_t made = 0;
        while (made < rp.W) {
            uint64_t G = lazy_budget(o, -1, rp.W - made);
            if (G == 0) {
                LT_TRY(spill_until(o, (uint64_t)o.P + 2 + 1, -1));
                G = lazy_budget(o, -1, rp.W - made);
                if (G == 0) return fail(LT_ERR_CAPACITY, "walker pool too small to create walkers");
            }
            LT_TRY(step_and_bucket(o, rp, -1, lazy_of(o, rp, -1, made, G), false, nullptr));
            made += G;
        }
    }
    refresh_all(o);
    return LT_OK;
}

// The scheduler loop of one run; stop = the run ended at a checkpoint.
lt_status run_loop(Ooc &o, const RunParams &rp, bool &stop)
{
    stop = false;
    if (o.policy->wave()) return wave_run(o, rp, stop);
    // Scheduler::start (src/Scheduler.h:425-438)
    bool sync = false;
    uint32_t p = 0;
    SchedView v = view(o);
    while (o.policy->next(v, o.prev_computed, sync, p)) {
        sync = false;
        do {
            LT_TRY(process(o, rp, p));
            LT_TRY(ckpt_point(o, rp, stop));
            if (stop) return LT_OK;
            v = view(o);
        } while (o.policy->next(v, o.prev_computed, false, p));
        sync = true;
        v = view(o);
    }
    return LT_OK;
}

// Device buffers and parameters of a call.
lt_status run_setup(lt_engine *e, RunParams &rp, int app, int start, uint32_t source, uint64_t W, uint32_t length,
                    float prob, bool endpoints, bool paths)
{
    Ooc &o = *e->ooc;
    lt_graph &g = *e->g;
    if (W >= (1ull << 32)) return fail(LT_ERR_INVALID, "out-of-core runs take fewer than 2^32 walkers per run");
    LT_TRY(ensure_pool(o, W));
    e->stats = lt_stats{};
    e->stats.cache_slots = o.K;
    e->stats.index_on_device = o.d_index != nullptr;
    std::fill(o.run_visits.begin(), o.run_visits.end(), 0);
    std::fill(o.run_cached_visits.begin(), o.run_cached_visits.end(), 0);
    std::fill(o.run_cached_launches.begin(), o.run_cached_launches.end(), 0);
    cudaStream_t st = e->s_compute;
    if (app != kWalk) LT_CUDA_TRY(cudaMemsetAsync(e->d_counts, 0, 8ull * g.V, st));
    LT_CUDA_TRY(cudaMemsetAsync(o.d_stats, 0, 64, st));
    if (endpoints) {
        LT_CUDA_TRY(cudaFree(e->d_endpoints));
        e->d_endpoints = nullptr;
        LT_TRY(dalloc(&e->d_endpoints, W));
    }
    if (paths) {
        LT_CUDA_TRY(cudaFree(e->d_paths));
        e->d_paths = nullptr;
        LT_TRY(dalloc(&e->d_paths, W * ((uint64_t)length + 1)));
    }
    rp = RunParams{};
    rp.app = app;
    rp.start = start;
    rp.source = source;
    rp.length = length;
    rp.W = W;
    rp.thr = app == kWalk ? 0 : threshold53(prob);
    rp.counts = app == kWalk ? nullptr : e->d_counts;
    rp.endpoints = endpoints ? e->d_endpoints : nullptr;
    rp.paths = paths ? e->d_paths : nullptr;
    return LT_OK;
}

// Runs run_index .. runs-1 (the first continuing from its queues when
// `resumed`), then the outputs.
lt_status run_all(lt_engine *e, RunParams &rp, uint32_t runs, uint32_t run_base, uint32_t first, bool resumed,
                  double t0, uint64_t *counts_out, uint32_t *endpoints_out, uint32_t *paths_out)
{
    Ooc &o = *e->ooc;
    lt_graph &g = *e->g;
    cudaStream_t st = e->s_compute;
    for (uint32_t r = first; r < runs; r++) {
        rp.run = run_base + r;
        o.run_index = r;
        if (!(resumed && r == first)) LT_TRY(run_prepare(o, rp));
        bool stop = false;
        LT_TRY(run_loop(o, rp, stop));
        if (stop) {
            LT_CUDA_TRY(cudaStreamSynchronize(st));
            LT_CUDA_TRY(cudaStreamSynchronize(e->s_copy));
            drain_timers(o, true);
            return fail(LT_INTERRUPTED, "run stopped at the checkpoint %s (iteration %llu)", o.ckpt_path.c_str(),
                        (unsigned long long)o.iteration);
        }
    }
    unsigned long long hs[8];
    LT_CUDA_TRY(cudaMemcpyAsync(hs, o.d_stats, sizeof hs, cudaMemcpyDeviceToHost, st));
    if (counts_out && rp.counts) LT_CUDA_TRY(cudaMemcpyAsync(counts_out, rp.counts, 8ull * g.V, cudaMemcpyDeviceToHost, st));
    if (endpoints_out && rp.endpoints)
        LT_CUDA_TRY(cudaMemcpyAsync(endpoints_out, rp.endpoints, 4 * rp.W, cudaMemcpyDeviceToHost, st));
    if (paths_out && rp.paths)
        LT_CUDA_TRY(cudaMemcpyAsync(paths_out, rp.paths, 4 * rp.W * ((uint64_t)rp.length + 1), cudaMemcpyDeviceToHost, st));
    LT_CUDA_TRY(cudaStreamSynchronize(st));
    LT_CUDA_TRY(cudaStreamSynchronize(e->s_copy));
    drain_timers(o, true);
    e->stats.updates = hs[0];
    e->stats.moves = hs[1];
    e->stats.teleports = hs[2];
    e->stats.zerocopy_bytes = hs[3] * zc_bytes_per_hop(o);
    e->stats.handoffs = hs[4];
    e->stats.running_ms = now_ms() - t0;
    // After the first run of a walk (PPR or PageRank, single source or any
    // start), the hot-vertex tier is built from its counts for the runs that
    // follow; outside the run's time.
    if (o.tier_bytes && !o.serve && rp.counts && (rp.app == kPPR || rp.app == kPageRank) &&
        !(o.tier_built && o.tier_app == rp.app && o.tier_start == rp.start && o.tier_source == rp.source)) {
        std::vector<uint64_t> tmp;
        const uint64_t *c = counts_out;
        if (!c) {
            tmp.resize(g.V);
            LT_CUDA_TRY(cudaMemcpy(tmp.data(), rp.counts, 8ull * g.V, cudaMemcpyDeviceToHost));
            c = tmp.data();
        }
        LT_TRY(tier_build(o, rp.app, rp.start, rp.source, c));
        e->stats.tier_build_ms = o.tier_build_ms;
    }
    return LT_OK;
}

}  // namespace

lt_status ooc_run(lt_engine *e, int app, int start, uint32_t source, uint64_t W, uint32_t length, uint32_t runs,
                  uint32_t run_base, float prob, uint64_t *counts_out, uint32_t *endpoints_out, uint32_t *paths_out)
{
    Ooc &o = *e->ooc;
    if (runs == 0) runs = 1;
    const double t0 = now_ms();
    RunParams rp;
    LT_TRY(run_setup(e, rp, app, start, source, W, length, prob, endpoints_out != nullptr, paths_out != nullptr));
    o.run_runs = runs;
    o.run_base = run_base;
    o.run_prob = prob;
    return run_all(e, rp, runs, run_base, 0, false, t0, counts_out, endpoints_out, paths_out);
}

lt_status ooc_checkpoint(Ooc *o, const char *path, uint64_t every, int stop)
{
    o->ckpt_path = path ? path : "";
    o->ckpt_every = path ? every : 0;
    o->ckpt_stop = stop != 0;
    return LT_OK;
}

lt_status checkpoint_info(const char *path, lt_checkpoint_info *out)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(LT_ERR_IO, "cannot open checkpoint %s", path);
    Reader r{f};
    CkptHeader h;
    const lt_status s = get_header(r, path, h);
    std::fclose(f);
    if (s != LT_OK) return s;
    out->app = (int)h.app;
    out->start_mode = (int)h.start;
    out->source = h.source;
    out->length = h.length;
    out->runs = h.runs;
    out->run_index = h.run_index;
    out->num_walkers = h.W;
    out->num_nodes = h.V;
    out->has_endpoints = (h.flags & 2u) ? 1 : 0;
    out->has_paths = (h.flags & 4u) ? 1 : 0;
    out->iteration = h.iteration;
    return LT_OK;
}

lt_status ooc_resume(lt_engine *e, const char *path, uint64_t *counts_out, uint32_t *endpoints_out, uint32_t *paths_out)
{
    Ooc &o = *e->ooc;
    lt_graph &g = *e->g;
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(LT_ERR_IO, "cannot open checkpoint %s", path);
    Reader r{f};
    CkptHeader h;
    lt_status s = get_header(r, path, h);
    if (s == LT_OK && (h.V != g.V || h.E != g.E || h.P != o.P))
        s = fail(LT_ERR_INVALID, "%s: checkpoint of another graph (V %u, E %llu, %u partitions)", path, h.V,
                 (unsigned long long)h.E, h.P);
    if (s == LT_OK && h.part_hash != part_table_hash(g))
        s = fail(LT_ERR_INVALID, "%s: checkpoint of other partition boundaries (partition size %llu here)", path,
                 (unsigned long long)g.part_bytes);
    const double t0 = now_ms();
    RunParams rp;
    if (s == LT_OK)
        s = run_setup(e, rp, (int)h.app, (int)h.start, h.source, h.W, h.length, h.prob, (h.flags & 2u) != 0,
                      (h.flags & 4u) != 0);
    unsigned long long hs[8];
    if (s == LT_OK) {
        r.get(hs, sizeof hs);
        std::vector<uint64_t> c;
        std::vector<uint32_t> v;
        if (rp.counts) {
            c.resize(g.V);
            r.get(c.data(), 8ull * g.V);
        }
        if (r.ok && rp.counts && cudaMemcpy(rp.counts, c.data(), 8ull * g.V, cudaMemcpyHostToDevice) != cudaSuccess)
            s = fail(LT_ERR_CUDA, "checkpoint upload failed");
        if (s == LT_OK && rp.endpoints) {
            v.resize(h.W);
            r.get(v.data(), 4ull * h.W);
            if (r.ok && cudaMemcpy(rp.endpoints, v.data(), 4ull * h.W, cudaMemcpyHostToDevice) != cudaSuccess)
                s = fail(LT_ERR_CUDA, "checkpoint upload failed");
        }
        if (s == LT_OK && rp.paths) {
            const uint64_t n = h.W * ((uint64_t)h.length + 1);
            v.resize(n);
            r.get(v.data(), 4ull * n);
            if (r.ok && cudaMemcpy(rp.paths, v.data(), 4ull * n, cudaMemcpyHostToDevice) != cudaSuccess)
                s = fail(LT_ERR_CUDA, "checkpoint upload failed");
        }
        if (s == LT_OK && !r.ok) s = fail(LT_ERR_FORMAT, "%s: truncated checkpoint", path);
        if (s == LT_OK && cudaMemcpy(o.d_stats, hs, sizeof hs, cudaMemcpyHostToDevice) != cudaSuccess)
            s = fail(LT_ERR_CUDA, "checkpoint upload failed");
    }
    if (s == LT_OK) {
        reset_queues(o);
        s = read_queues(o, r, path, h);
    }
    std::fclose(f);
    if (s != LT_OK) {
        reset_queues(o);
        refresh_all(o);
        return s;
    }
    refresh_all(o);
    o.prev_computed = -1;
    o.run_runs = h.runs;
    o.run_base = h.run_base;
    o.run_prob = h.prob;
    o.iteration = h.iteration;
    // the walks continue with the checkpoint's random stream
    const uint64_t seed = e->cfg.seed;
    e->cfg.seed = h.seed;
    s = run_all(e, rp, h.runs, h.run_base, h.run_index, true, t0, counts_out, endpoints_out, paths_out);
    e->cfg.seed = seed;
    return s;
}

}  // namespace lt

// ===========================================================================
// Serving: continuous batching of PPR queries on the out-of-core engine.
//
// A query (source, walkers, seed) is admitted when a query slot, room in the
// per-query table arena and walker-pool chunks for all its walkers are free
// (admission by free device memory); its walkers are written straight into
// its source partition's queue and from then on share every scheduler
// iteration, cache slot and kernel launch with the queries already running.
// Walker state stays in the device pool (spilled only under pressure).  Each
// walker draws from its query's key and index, so a query's counts do not
// depend on what else runs.  After every iteration the finished-walker
// counters of the active queries come back to the host; a query whose count
// reached its walker total is extracted (its table compacted on the device)
// and its slot, table and chunks are released.
// ===========================================================================

struct lt_server {
    struct Query {
        uint64_t ticket = 0;
        uint32_t source = 0;
        uint64_t walkers = 0, seed = 0;
        int32_t slot = -1;
        uint64_t toff = 0;
        uint32_t tlog = 0;
        double t_arrive = 0, t_done = 0;
        int state = 0;  // 0 pending, 1 active, 2 done
        std::vector<uint32_t> out_v, out_c;
    };
    lt_engine *e = nullptr;
    lt::WaveState *wave = nullptr;  // wave-run policies: one wave iteration per serving step
    lt::Ooc *o = nullptr;
    uint32_t max_active = 0;
    uint64_t table_cap = 0;
    float prob = 0.15f;
    uint64_t thr = 0;
    uint64_t *d_seed = nullptr, *d_toff = nullptr;
    uint32_t *d_tlog = nullptr, *d_keys = nullptr, *d_cnt = nullptr;
    unsigned long long *d_done = nullptr, *d_err = nullptr, *d_outn = nullptr;
    uint32_t *d_out_v = nullptr, *d_out_c = nullptr;
    uint64_t out_cap = 0;
    uint64_t *d_meta = nullptr;  // extraction metadata: table base, size, output base and count per finished query
    lt::HostBuf h_done;
    std::vector<Query *> slots;
    std::deque<Query *> pending;
    std::map<uint64_t, Query *> all;
    uint64_t next_ticket = 1;
    std::vector<std::vector<uint64_t>> free_by_log;  // table arena free list per size class
    uint64_t bump = 0;
    uint64_t live_walkers = 0;
    std::vector<uint64_t> finished;  // tickets completed since the last drain
};

namespace lt {

double serve_now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

namespace {

__global__ void serve_slot_kernel(uint64_t *seed, uint64_t *toff, uint32_t *tlog, unsigned long long *done,
                                  uint32_t slot, uint64_t sv, uint64_t tv, uint32_t lv)
{
    seed[slot] = sv;
    toff[slot] = tv;
    tlog[slot] = lv;
    done[slot] = 0;
}

__global__ void serve_clear_kernel(uint32_t *keys, uint32_t *cnt, uint64_t base, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        keys[base + i] = 0xFFFFFFFFu;
        cnt[base + i] = 0;
    }
}

// One CTA per finished query: its occupied table slots become (vertex, count)
// pairs at out + obase[k].
__global__ void serve_extract_kernel(const uint32_t *keys, const uint32_t *cnt, const uint64_t *tbase,
                                     const uint64_t *tsize, const uint64_t *obase, unsigned long long *outn,
                                     uint32_t *out_v, uint32_t *out_c)
{
    const uint32_t k = blockIdx.x;
    const uint64_t b = tbase[k], n = tsize[k], o = obase[k];
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t key = keys[b + i];
        if (key != 0xFFFFFFFFu) {
            const unsigned long long pos = atomicAdd(&outn[k], 1ull);
            out_v[o + pos] = key;
            out_c[o + pos] = cnt[b + i];
        }
    }
}

void serve_args(Ooc &o, StepArgs &a)
{
    lt_server &s = *o.serve;
    a.q_seed = s.d_seed;
    a.q_toff = s.d_toff;
    a.q_tlog = s.d_tlog;
    a.q_keys = s.d_keys;
    a.q_cnt = s.d_cnt;
    a.q_done = s.d_done;
    a.q_error = s.d_err;
}

bool table_alloc(lt_server &s, uint32_t lg, uint64_t &off)
{
    if (lg < s.free_by_log.size() && !s.free_by_log[lg].empty()) {
        off = s.free_by_log[lg].back();
        s.free_by_log[lg].pop_back();
        return true;
    }
    const uint64_t size = 1ull << lg;
    const uint64_t aligned = (s.bump + size - 1) & ~(size - 1);
    if (aligned + size > s.table_cap) return false;
    off = aligned;
    s.bump = aligned + size;
    return true;
}

void table_free(lt_server &s, uint32_t lg, uint64_t off)
{
    if (s.free_by_log.size() <= lg) s.free_by_log.resize(lg + 1);
    s.free_by_log[lg].push_back(off);
}

uint32_t log2_ceil_host(uint64_t x)
{
    uint32_t l = 0;
    while ((1ull << l) < x) l++;
    return l;
}

// Admit pending queries while a slot, table room and walker chunks are free.
lt_status serve_admit(lt_server &s)
{
    Ooc &o = *s.o;
    lt_engine &e = *s.e;
    lt_graph &g = *o.g;
    while (!s.pending.empty()) {
        lt_server::Query *q = s.pending.front();
        int32_t slot = -1;
        for (uint32_t i = 0; i < s.max_active; i++)
            if (!s.slots[i]) {
                slot = (int32_t)i;
                break;
            }
        if (slot < 0) break;
        const uint32_t p = g.find_partition(q->source);
        Queue &qp = o.q[p];
        const bool open_tail = !qp.dev_chunks.empty() && qp.tail_fill < kChunk;
        const uint64_t fill = open_tail ? qp.tail_fill : 0;
        const uint64_t need = (fill + q->walkers + kChunk - 1) / kChunk - (open_tail ? 1 : 0);
        if (o.free_chunks.size() < need + (uint64_t)o.P + 2) break;  // keep room for the walkers to move
        const uint32_t lg = std::max<uint32_t>(5, log2_ceil_host(q->walkers * 2));
        uint64_t toff = 0;
        if (!table_alloc(s, lg, toff)) break;
        s.pending.pop_front();
        q->slot = slot;
        q->toff = toff;
        q->tlog = lg;
        q->state = 1;
        s.slots[slot] = q;
        s.live_walkers += q->walkers;
        serve_slot_kernel<<<1, 1, 0, e.s_compute>>>(s.d_seed, s.d_toff, s.d_tlog, s.d_done, (uint32_t)slot, q->seed,
                                                   toff, lg);
        serve_clear_kernel<<<std::max<uint64_t>(1, std::min<uint64_t>((1ull << lg) / 256, 256)), 256, 0,
                             e.s_compute>>>(s.d_keys, s.d_cnt, toff, 1ull << lg);
        // append the walkers to the source partition's queue
        if (qp.dev_chunks.empty() || qp.tail_fill == kChunk) {
            qp.dev_chunks.push_back(o.free_chunks.back());
            o.free_chunks.pop_back();
            qp.tail_fill = 0;
        }
        uint32_t *h_chunks = (uint32_t *)o.h_plan.ptr;
        uint64_t n_plan = 0;
        h_chunks[n_plan++] = qp.dev_chunks.back();
        const uint32_t cursor = qp.tail_fill;
        const uint64_t tot = (uint64_t)qp.tail_fill + q->walkers;
        const uint64_t extra = (tot + kChunk - 1) / kChunk - 1;
        for (uint64_t k = 0; k < extra; k++) {
            const uint32_t c = o.free_chunks.back();
            o.free_chunks.pop_back();
            qp.dev_chunks.push_back(c);
            h_chunks[n_plan++] = c;
        }
        qp.tail_fill = (uint32_t)(tot - extra * kChunk);
        LT_CUDA_TRY(cudaMemcpyAsync(o.d_planbuf, h_chunks, 4 * n_plan, cudaMemcpyHostToDevice, e.s_compute));
        InjectArgs ia{};
        ia.arena = o.d_arena;
        ia.plan_chunks = o.d_planbuf;
        ia.cursor = cursor;
        ia.n = q->walkers;
        ia.source = q->source;
        ia.qslot = (uint32_t)slot;
        ia.seed = q->seed;
        ia.thr = s.thr;
        LT_CUDA_TRY(launch_inject(ia, e.device, e.s_compute));
        // the pinned plan block is rewritten by the next admission: let the copy finish
        LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
        refresh(o, p);
    }
    return LT_OK;
}

// Extract every active query whose walkers have all finished.
lt_status serve_complete(lt_server &s, uint32_t &completed)
{
    Ooc &o = *s.o;
    lt_engine &e = *s.e;
    completed = 0;
    unsigned long long *h_done = (unsigned long long *)s.h_done.ptr;
    LT_CUDA_TRY(cudaMemcpyAsync(h_done, s.d_done, 8ull * s.max_active, cudaMemcpyDeviceToHost, e.s_compute));
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    std::vector<lt_server::Query *> fin;
    for (uint32_t i = 0; i < s.max_active; i++)
        if (s.slots[i] && h_done[i] >= s.slots[i]->walkers) fin.push_back(s.slots[i]);
    if (fin.empty()) return LT_OK;
    std::vector<uint64_t> meta(3 * fin.size());
    uint64_t obase = 0;
    for (size_t k = 0; k < fin.size(); k++) {
        meta[k] = fin[k]->toff;
        meta[fin.size() + k] = 1ull << fin[k]->tlog;
        meta[2 * fin.size() + k] = obase;
        obase += fin[k]->walkers;
    }
    if (obase > s.out_cap) {
        // the output staging grows geometrically (rarely: to the largest
        // batch of finished walkers seen so far)
        for (void *p : {(void *)s.d_out_v, (void *)s.d_out_c})
            if (p) cudaFree(p);
        s.out_cap = std::max<uint64_t>(obase, 2 * s.out_cap);
        LT_CUDA_TRY(cudaMalloc(&s.d_out_v, 4 * s.out_cap));
        LT_CUDA_TRY(cudaMalloc(&s.d_out_c, 4 * s.out_cap));
    }
    // at most max_active queries finish in one step: the metadata block
    // allocated at serve_open always holds them
    uint64_t *d_meta = s.d_meta;
    unsigned long long *d_n = (unsigned long long *)(d_meta + meta.size());
    LT_CUDA_TRY(cudaMemcpyAsync(d_meta, meta.data(), 8 * meta.size(), cudaMemcpyHostToDevice, e.s_compute));
    LT_CUDA_TRY(cudaMemsetAsync(d_n, 0, 8 * fin.size(), e.s_compute));
    serve_extract_kernel<<<(unsigned)fin.size(), 256, 0, e.s_compute>>>(s.d_keys, s.d_cnt, d_meta, d_meta + fin.size(),
                                                                          d_meta + 2 * fin.size(), d_n, s.d_out_v,
                                                                          s.d_out_c);
    LT_CUDA_TRY(cudaGetLastError());
    std::vector<unsigned long long> nn(fin.size());
    LT_CUDA_TRY(cudaMemcpyAsync(nn.data(), d_n, 8 * fin.size(), cudaMemcpyDeviceToHost, e.s_compute));
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    const double now = serve_now_ms();
    for (size_t k = 0; k < fin.size(); k++) {
        lt_server::Query *q = fin[k];
        q->out_v.resize(nn[k]);
        q->out_c.resize(nn[k]);
        LT_CUDA_TRY(cudaMemcpyAsync(q->out_v.data(), s.d_out_v + meta[2 * fin.size() + k], 4 * nn[k],
                                    cudaMemcpyDeviceToHost, e.s_compute));
        LT_CUDA_TRY(cudaMemcpyAsync(q->out_c.data(), s.d_out_c + meta[2 * fin.size() + k], 4 * nn[k],
                                    cudaMemcpyDeviceToHost, e.s_compute));
    }
    LT_CUDA_TRY(cudaStreamSynchronize(e.s_compute));
    for (lt_server::Query *q : fin) {
        q->state = 2;
        q->t_done = now;
        s.finished.push_back(q->ticket);
        s.slots[q->slot] = nullptr;
        table_free(s, q->tlog, q->toff);
        s.live_walkers -= q->walkers;
        completed++;
    }
    (void)o;
    return LT_OK;
}

}  // namespace

lt_status serve_open(lt_engine *e, uint32_t max_active, uint64_t table_slots, float prob, lt_server **out)
{
    if (!e->ooc) return fail(LT_ERR_UNSUPPORTED, "serving runs on the out-of-core engine (-p below the partition count)");
    if (e->ooc->serve) return fail(LT_ERR_INVALID, "the engine already serves");
    if (!(prob > 0.0f && prob <= 1.0f)) return fail(LT_ERR_INVALID, "PPR stop probability must be in (0, 1]");
    if (max_active == 0 || table_slots < 64) return fail(LT_ERR_INVALID, "no room for queries");
    LT_CUDA_TRY(cudaSetDevice(e->device));
    Ooc &o = *e->ooc;
    LT_TRY(ensure_pool(o, e->cfg.num_device_walkers ? e->cfg.num_device_walkers : (1ull << 26)));
    lt_server *s = new lt_server();
    s->e = e;
    s->o = &o;
    s->max_active = max_active;
    s->table_cap = table_slots;
    s->prob = prob;
    s->thr = threshold53(prob);
    s->slots.assign(max_active, nullptr);
    auto bail = [&](lt_status st) {
        serve_close(s);
        return st;
    };
    lt_status st = dalloc(&s->d_seed, max_active);
    if (st == LT_OK) st = dalloc(&s->d_toff, max_active);
    if (st == LT_OK) st = dalloc(&s->d_tlog, max_active);
    if (st == LT_OK) st = dalloc(&s->d_done, max_active);
    if (st == LT_OK) st = dalloc(&s->d_err, 1);
    if (st == LT_OK) st = dalloc(&s->d_keys, table_slots);
    if (st == LT_OK) st = dalloc(&s->d_cnt, table_slots);
    if (st == LT_OK) st = dalloc(&s->d_meta, 4ull * max_active);
    if (st == LT_OK) st = host_alloc(s->h_done, 8ull * max_active, true);
    if (st != LT_OK) return bail(st);
    if (cudaMemset(s->d_done, 0, 8ull * max_active) != cudaSuccess || cudaMemset(s->d_err, 0, 8) != cudaSuccess)
        return bail(fail(LT_ERR_CUDA, "serving state initialisation failed"));
    reset_queues(o);
    refresh_all(o);
    cudaMemsetAsync(o.d_stats, 0, 64, e->s_compute);
    e->stats = lt_stats{};
    e->stats.cache_slots = o.K;
    e->stats.index_on_device = o.d_index != nullptr;
    o.serve = s;
    if (o.policy->wave()) s->wave = new WaveState(o.P);
    *out = s;
    return LT_OK;
}

lt_status serve_submit(lt_server *s, uint32_t source, uint64_t walkers, uint64_t seed, double arrival_ms, uint64_t *ticket)
{
    if (source >= s->o->g->V) return fail(LT_ERR_INVALID, "source %u out of range", source);
    if (walkers == 0 || walkers >= (1ull << 32)) return fail(LT_ERR_INVALID, "walkers must be in [1, 2^32)");
    auto *q = new lt_server::Query();
    q->ticket = s->next_ticket++;
    q->source = source;
    q->walkers = walkers;
    q->seed = seed;
    q->t_arrive = arrival_ms > 0 ? arrival_ms : serve_now_ms();
    s->pending.push_back(q);
    s->all[q->ticket] = q;
    *ticket = q->ticket;
    return LT_OK;
}

lt_status serve_step(lt_server *s, uint32_t *completed, uint32_t *active, uint32_t *pending)
{
    Ooc &o = *s->o;
    lt_engine &e = *s->e;
    LT_CUDA_TRY(cudaSetDevice(e.device));
    LT_TRY(serve_admit(*s));
    uint32_t p = 0;
    SchedView v = view(o);
    if (s->wave) {
        // light load: every step is a final sweep that finishes the admitted
        // walkers in one kernel; heavy load: waves with overlapped loads
        RunParams rp{};
        rp.app = kPPR;
        rp.start = kStartSource;
        rp.thr = s->thr;
        bool idle = false;
        LT_TRY(wave_step(o, rp, *s->wave, idle));
    } else if (o.policy->next(v, o.prev_computed, false, p) || o.policy->next(v, o.prev_computed, true, p)) {
        RunParams rp{};
        rp.app = kPPR;
        rp.start = kStartSource;
        rp.thr = s->thr;
        rp.W = 0;
        LT_TRY(process(o, rp, p));
    }
    uint32_t done = 0;
    LT_TRY(serve_complete(*s, done));
    if (completed) *completed = done;
    uint32_t act = 0;
    for (lt_server::Query *q : s->slots) act += q != nullptr;
    if (active) *active = act;
    if (pending) *pending = (uint32_t)s->pending.size();
    return LT_OK;
}

lt_status serve_result(lt_server *s, uint64_t ticket, int *done, uint64_t *n_pairs, uint32_t *vertices,
                       uint32_t *counts, uint64_t capacity, double *latency_ms)
{
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return fail(LT_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
    lt_server::Query *q = it->second;
    if (done) *done = q->state == 2;
    if (q->state != 2) return LT_OK;
    if (n_pairs) *n_pairs = q->out_v.size();
    if (latency_ms) *latency_ms = q->t_done - q->t_arrive;
    if (vertices && counts) {
        if (capacity < q->out_v.size()) return fail(LT_ERR_CAPACITY, "result has %zu pairs", q->out_v.size());
        std::memcpy(vertices, q->out_v.data(), 4 * q->out_v.size());
        std::memcpy(counts, q->out_c.data(), 4 * q->out_c.size());
        s->all.erase(it);
        delete q;
    }
    return LT_OK;
}

uint64_t serve_finished(lt_server *s, uint64_t *tickets, uint64_t cap)
{
    const uint64_t n = std::min<uint64_t>(cap, s->finished.size());
    if (tickets) std::memcpy(tickets, s->finished.data(), 8 * n);
    s->finished.erase(s->finished.begin(), s->finished.begin() + n);
    return n;
}

void serve_close(lt_server *s)
{
    if (!s) return;
    if (s->o && s->o->serve == s) {
        cudaStreamSynchronize(s->e->s_compute);
        unsigned long long hs[8];
        if (cudaMemcpy(hs, s->o->d_stats, sizeof hs, cudaMemcpyDeviceToHost) == cudaSuccess) {
            s->e->stats.updates = hs[0];
            s->e->stats.moves = hs[1];
            s->e->stats.teleports = hs[2];
            s->e->stats.zerocopy_bytes = hs[3] * zc_bytes_per_hop(*s->o);
            s->e->stats.handoffs = hs[4];
        }
        if (s->wave) {
            // loads still in flight: let them land and publish them
            cudaStreamSynchronize(s->e->s_copy);
            for (auto &d : s->wave->inflight) set_entry(*s->o, d.first, s->e->s_compute);
            cudaStreamSynchronize(s->e->s_compute);
        }
        drain_timers(*s->o, true);
        s->o->serve = nullptr;
        reset_queues(*s->o);
        refresh_all(*s->o);
    }
    for (void *p : {(void *)s->d_seed, (void *)s->d_toff, (void *)s->d_tlog, (void *)s->d_keys, (void *)s->d_cnt,
                    (void *)s->d_done, (void *)s->d_err, (void *)s->d_out_v, (void *)s->d_out_c, (void *)s->d_meta})
        if (p) cudaFree(p);
    host_free(s->h_done);
    delete s->wave;
    for (auto &kv : s->all) delete kv.second;
    for (lt_server::Query *q : s->pending)
        if (s->all.find(q->ticket) == s->all.end()) delete q;
    delete s;
}

}  // namespace lt
