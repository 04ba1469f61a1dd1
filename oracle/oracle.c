/*
 * oracle/oracle.c -- CPU restatement of LightTraffic's random-walk semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA product
 * is compared against.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it.  Nothing in the
 * product links, loads or calls it.
 *
 * What it restates (reference paths relative to the LightTraffic project):
 *   - PPR        app/ppr.cu:22-42 (App::update) + src/walk/SingleSource.h:11-18
 *                (geometric walk length, "step = 2; while (U > prob) step++").
 *   - PageRank   app/pagerank.cu:26-44 (App::update, alpha = 0.85 at
 *                app/pagerank.cu:6) + src/walk/NodeSampler.h:10-13 (uniform
 *                start).  The reference computes "% 0" on a vertex with no
 *                out-edges (undefined behaviour); here such a walker teleports.
 *   - generic    app/genericwalk.cu:22-32 (move to a uniform neighbour, stop at
 *     walk       a vertex with no out-edges).  Paths follow the layout of
 *                src/walk/NodeSampler.h:31-49 (INVALID_NODE = 0xFFFFFFFF padding,
 *                src/Type.h:18), with l+1 entries per walk (source + l hops).
 *   - integer draw  src/Rand.h:17-19: uniform_discrete(n) = (hi<<32 | lo) % n.
 *   - "walk while inside the partition" (src/WalkManager.h:239-240): because
 *     every draw below is keyed by (seed, run, walker index, step value) and
 *     never by thread or schedule, walking a walker to completion over the
 *     whole graph gives the same result as any partition-by-partition order.
 *
 * The reference draws from cuRAND XORWOW with per-thread state and an
 * uninitialised seed (src/Rand.h:29-30), so its own outputs are not
 * reproducible.  Both this oracle and the product replace it with
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As
 * Easy as 1, 2, 3", SC 2011), keyed per walker:
 *
 *   key     = (seed & 0xffffffff, seed >> 32)
 *   counter = (c0, tag | run << 8, idx & 0xffffffff, idx >> 32)
 *     init draws  : tag 1, c0 = draw number t (0, 1, 2, ...)
 *     step draws  : tag 2, c0 = walker.step before the update
 *   r64   = x0 << 32 | x1            (neighbour / vertex choice, r64 % n)
 *   m53   = (x2 << 32 | x3) >> 11    (uniform double U = (m53 + 1) * 2^-53,
 *                                     so U lies in (0, 1] like
 *                                     curand_uniform_double)
 *   "U > p"  <=>  m53 >= floor(p * 2^53)   (exact; p is a float widened to
 *                                           double, as in the reference)
 *   PPR length trials: init draw t gives two trials, m53 of (x0,x1) first,
 *   then m53 of (x2,x3).
 *
 * Pinning.  Walk semantics: the reference's own update code is the pin.
 * oracle/ref_apps_main.cpp compiles app/ppr.cu, app/pagerank.cu and
 * app/genericwalk.cu in place with g++ (host stand-ins for their GPU
 * plumbing in oracle/ref_shim/) and drives their App::update partition by
 * partition, as src/WalkManager.h:229-246 does, with the keyed stream above
 * in place of cuRAND; its outputs (tests/golden/ref_walks.json) must equal
 * this file's bit for bit (tests/test_ref_pin.py).  The reference's cuRAND
 * streams themselves are not reproducible (uninitialised seed), so they are
 * not the target.  Also pinned: the sum invariants (PPR counts sum to the
 * number of walkers, app/ppr.cu:77-85; PageRank to walkers x length x runs,
 * app/pagerank.cu:89-97), hand-checkable graphs, Philox against the
 * Random123 known-answer vectors, and the partitioner (orc_partition) byte
 * for byte against the reference's EqualSizeStrategy compiled from its own
 * sources.
 *
 * The RMAT generator (a seeded stand-in for the reference's datasets, which
 * are absent) is restated here as well so the GPU generator can be checked
 * bit-exact:
 *   source of edge i: level l (0 = most significant bit) uses 16-bit lane l
 *     of Philox(ctr = (i lo, i hi, 0x10, l / 8), key = seed); lanes are taken
 *     x0 low half, x0 high half, x1 low, x1 high, ... ; bit = lane >= T_src.
 *   destination of the k-th out-edge of u: lane l of
 *     Philox(ctr = (u, k, 0x11, l / 8)); bit = lane >= (bit_l(u) ? T_d1 : T_d0).
 *   Isolated vertices (no in- and no out-edges) are removed keeping order,
 *   following tools/rm_isolated_vertices.cc:70-87.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <omp.h>

#define ORC_TAG_INIT 1u
#define ORC_TAG_STEP 2u
#define ORC_TAG_RMAT_SRC 0x10u
#define ORC_TAG_RMAT_DST 0x11u
#define ORC_INVALID_NODE 0xFFFFFFFFu

enum { ORC_APP_PPR = 0, ORC_APP_PAGERANK = 1, ORC_APP_WALK = 2 };
enum { ORC_START_SOURCE = 0, ORC_START_UNIFORM = 1, ORC_START_PER_VERTEX = 2 };

/* ---------------------------------------------------------------- Philox */

static void orc_philox_impl(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        if (r > 0) { k0 += W0; k1 += W1; }
        uint64_t p0 = (uint64_t)M0 * (uint64_t)c0;
        uint64_t p1 = (uint64_t)M1 * (uint64_t)c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

int orc_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out)
{
    orc_philox_impl(ctr, key, out);
    return 0;
}

static inline void walk_draw(uint64_t seed, uint32_t c0, uint32_t tag, uint32_t run,
                             uint64_t idx, uint32_t x[4])
{
    uint32_t ctr[4] = { c0, tag | (run << 8), (uint32_t)idx, (uint32_t)(idx >> 32) };
    uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
    orc_philox_impl(ctr, key, x);
}

/* floor(p * 2^53) for a float p in [0, 1], computed exactly (scaling by a
 * power of two is exact in double). */
uint64_t orc_threshold53(float p)
{
    double d = (double)p;
    if (!(d > 0.0)) return 0;
    if (d >= 1.0) return (uint64_t)1 << 53;
    return (uint64_t)(d * 9007199254740992.0);
}

/* ------------------------------------------------------------------ walks */

/* Walk length of PPR walker idx: src/walk/SingleSource.h:11-18. */
uint32_t orc_ppr_length(uint64_t seed, uint32_t run, uint64_t idx, uint64_t thr)
{
    uint32_t step = 2;
    for (uint32_t t = 0;; t++) {
        uint32_t x[4];
        walk_draw(seed, t, ORC_TAG_INIT, run, idx, x);
        uint64_t m0 = (((uint64_t)x[0] << 32) | x[1]) >> 11;
        if (m0 < thr) return step;
        step++;
        uint64_t m1 = (((uint64_t)x[2] << 32) | x[3]) >> 11;
        if (m1 < thr) return step;
        step++;
    }
}

static uint32_t start_vertex(int start_mode, uint32_t source, uint32_t V, uint64_t seed,
                             uint32_t run, uint64_t idx)
{
    if (start_mode == ORC_START_SOURCE) return source;
    if (start_mode == ORC_START_PER_VERTEX) return (uint32_t)(idx % V);
    uint32_t x[4];
    walk_draw(seed, 0, ORC_TAG_INIT, run, idx, x);
    uint64_t r64 = ((uint64_t)x[0] << 32) | x[1];
    return (uint32_t)(r64 % V);
}

/*
 * Run one batch of W walkers of the given app and accumulate into the outputs.
 *   counts   : u64[V], added to (PPR endpoint counts / PageRank visit counts)
 *   endpoints: u32[W] or NULL (final vertex of each walker)
 *   paths    : u32[W * (length + 1)] or NULL (generic walk only)
 *   stats    : u64[3] or NULL: {updates, graph moves (hops), teleports}
 */
int orc_walk_batch(int app, uint32_t V, const uint64_t *rowptr, const uint32_t *col,
                   int start_mode, uint32_t source, uint64_t W, uint32_t length,
                   float prob, uint32_t run, uint64_t seed,
                   uint64_t *counts, uint32_t *endpoints, uint32_t *paths,
                   uint64_t *stats, int threads)
{
    if (V == 0 || (app == ORC_APP_PPR && !(prob > 0.0f))) return -1;
    if (app != ORC_APP_PPR && length == 0) return -1;
    uint64_t thr = orc_threshold53(prob);
    uint64_t tot_updates = 0, tot_moves = 0, tot_tele = 0;
    if (threads <= 0) threads = omp_get_max_threads();

#pragma omp parallel for schedule(dynamic, 4096) num_threads(threads) \
    reduction(+ : tot_updates, tot_moves, tot_tele)
    for (int64_t si = 0; si < (int64_t)W; si++) {
        uint64_t idx = (uint64_t)si;
        uint32_t cur = start_vertex(start_mode, source, V, seed, run, idx);
        uint32_t step = (app == ORC_APP_PPR) ? orc_ppr_length(seed, run, idx, thr) : length;
        uint32_t *path = NULL;
        if (paths) {
            path = paths + idx * (uint64_t)(length + 1);
            path[0] = cur;
        }
        uint64_t updates = 0, moves = 0, tele = 0;
        while (step > 0) {
            uint32_t s = step;
            updates++;
            if (app == ORC_APP_PPR) {
                /* app/ppr.cu:22-42 */
                if (step == 1) {
                    __atomic_fetch_add(&counts[cur], 1, __ATOMIC_RELAXED);
                }
                step -= 1;
                if (step == 0) break;
                uint64_t first = rowptr[cur];
                uint64_t deg = rowptr[cur + 1] - first;
                if (deg > 0) {
                    uint32_t x[4];
                    walk_draw(seed, s, ORC_TAG_STEP, run, idx, x);
                    uint64_t r64 = ((uint64_t)x[0] << 32) | x[1];
                    cur = col[first + r64 % deg];
                    moves++;
                } else {
                    __atomic_fetch_add(&counts[cur], 1, __ATOMIC_RELAXED);
                    step = 0;
                }
            } else if (app == ORC_APP_PAGERANK) {
                /* app/pagerank.cu:26-44 */
                __atomic_fetch_add(&counts[cur], 1, __ATOMIC_RELAXED);
                step -= 1;
                if (step == 0) break;
                uint32_t x[4];
                walk_draw(seed, s, ORC_TAG_STEP, run, idx, x);
                uint64_t r64 = ((uint64_t)x[0] << 32) | x[1];
                uint64_t m53 = (((uint64_t)x[2] << 32) | x[3]) >> 11;
                uint64_t first = rowptr[cur];
                uint64_t deg = rowptr[cur + 1] - first;
                if (m53 >= thr || deg == 0) {
                    cur = (uint32_t)(r64 % V);
                    tele++;
                } else {
                    cur = col[first + r64 % deg];
                    moves++;
                }
            } else {
                /* app/genericwalk.cu:22-32 */
                uint64_t first = rowptr[cur];
                uint64_t deg = rowptr[cur + 1] - first;
                if (deg > 0) {
                    uint32_t x[4];
                    walk_draw(seed, s, ORC_TAG_STEP, run, idx, x);
                    uint64_t r64 = ((uint64_t)x[0] << 32) | x[1];
                    cur = col[first + r64 % deg];
                    moves++;
                    if (path) path[length - s + 1] = cur;
                } else {
                    step = 1;
                    if (path) {
                        for (uint32_t h = length - s + 1; h <= length; h++) path[h] = ORC_INVALID_NODE;
                    }
                }
                step -= 1;
            }
        }
        if (endpoints) endpoints[idx] = cur;
        tot_updates += updates;
        tot_moves += moves;
        tot_tele += tele;
    }
    if (stats) {
        stats[0] += tot_updates;
        stats[1] += tot_moves;
        stats[2] += tot_tele;
    }
    return 0;
}

/* ------------------------------------------------------------- partitioner */

/*
 * Greedy vertex-range partitioner, restating EqualSizeStrategy::init
 * (src/partition/PartitionStrategy.h:189-218): a partition [n, i) is grown
 * while (i - n + 1) * 8 + (rowptr[i] - rowptr[n]) * 4 <= max_bytes; when the
 * test fails with i > n + 1 the partition is closed at i - 1 and the test is
 * repeated for the same i against the new start; a single vertex that does
 * not fit is an error (return -2).  Returns the partition count in *num_parts,
 * or -3 if more than cap partitions would be produced.
 */
int orc_partition(const uint64_t *rowptr, uint32_t V, uint64_t max_bytes,
                  uint32_t *node_off, uint64_t *edge_off, uint32_t cap, uint32_t *num_parts)
{
    uint32_t n = 0, P = 0;
    if (cap < 1) return -3;
    node_off[0] = 0;
    edge_off[0] = 0;
    for (uint32_t i = 1; i <= V;) {
        uint64_t size = (uint64_t)(i - n + 1) * 8u + (rowptr[i] - rowptr[n]) * 4u;
        if (size > max_bytes) {
            if (i == n + 1) return -2;
            n = i - 1;
            P++;
            if (P + 1 > cap) return -3;
            node_off[P] = n;
            edge_off[P] = rowptr[n];
        } else {
            i++;
        }
    }
    P++;
    if (P + 1 > cap) return -3;
    node_off[P] = V;
    edge_off[P] = rowptr[V];
    *num_parts = P;
    return 0;
}

/* ------------------------------------------------------------------- RMAT */

static inline uint32_t lane16(const uint32_t x[4], int l)
{
    uint32_t w = x[l >> 1];
    return (l & 1) ? (w >> 16) : (w & 0xFFFFu);
}

static uint32_t rmat_src(uint64_t seed, uint64_t i, int scale, uint32_t t_src)
{
    uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
    uint32_t v = 0, x[4];
    for (int l = 0; l < scale; l++) {
        if ((l & 7) == 0) {
            uint32_t ctr[4] = { (uint32_t)i, (uint32_t)(i >> 32), ORC_TAG_RMAT_SRC, (uint32_t)(l >> 3) };
            orc_philox_impl(ctr, key, x);
        }
        uint32_t bit = lane16(x, l & 7) >= t_src;
        v = (v << 1) | bit;
    }
    return v;
}

static uint32_t rmat_dst(uint64_t seed, uint32_t u, uint32_t k, int scale, uint32_t t_d0, uint32_t t_d1)
{
    uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
    uint32_t v = 0, x[4];
    for (int l = 0; l < scale; l++) {
        if ((l & 7) == 0) {
            uint32_t ctr[4] = { u, k, ORC_TAG_RMAT_DST, (uint32_t)(l >> 3) };
            orc_philox_impl(ctr, key, x);
        }
        uint32_t sbit = (u >> (scale - 1 - l)) & 1u;
        uint32_t bit = lane16(x, l & 7) >= (sbit ? t_d1 : t_d0);
        v = (v << 1) | bit;
    }
    return v;
}

/*
 * Phase 1: out-degrees of the 2^scale raw vertices (deg: u64[2^scale]).
 */
int orc_rmat_degrees(int scale, uint64_t E, uint64_t seed, uint32_t t_src, uint64_t *deg, int threads)
{
    uint64_t V0 = (uint64_t)1 << scale;
    if (threads <= 0) threads = omp_get_max_threads();
    memset(deg, 0, V0 * sizeof(uint64_t));
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t i = 0; i < (int64_t)E; i++) {
        uint32_t s = rmat_src(seed, (uint64_t)i, scale, t_src);
        __atomic_fetch_add(&deg[s], 1, __ATOMIC_RELAXED);
    }
    return 0;
}

/*
 * Phase 2: given raw rowptr (u64[2^scale + 1]), fill raw col (u32[E]).
 */
int orc_rmat_fill(int scale, uint64_t seed, uint32_t t_d0, uint32_t t_d1,
                  const uint64_t *rowptr, uint32_t *col, int threads)
{
    uint64_t V0 = (uint64_t)1 << scale;
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads)
    for (int64_t u = 0; u < (int64_t)V0; u++) {
        uint64_t b = rowptr[u], e = rowptr[u + 1];
        for (uint64_t k = 0; k < e - b; k++) {
            col[b + k] = rmat_dst(seed, (uint32_t)u, (uint32_t)k, scale, t_d0, t_d1);
        }
    }
    return 0;
}

/*
 * Phase 3: remove isolated raw vertices (no out-edges and never a
 * destination), keeping order (tools/rm_isolated_vertices.cc:70-87).
 *   rowptr : raw u64[V0 + 1] from the degrees
 *   col    : raw u32[E], rewritten in place to the compacted ids
 *   newid  : scratch u32[V0]; present : scratch u8[V0]
 *   out_rp : u64[V0 + 1], not aliasing rowptr; its first *out_V + 1 entries
 *            are the compacted rowptr (an isolated vertex has no edges, so a
 *            kept vertex keeps its raw edge offset)
 */
int orc_rmat_compact(uint64_t V0, uint64_t E, const uint64_t *rowptr, uint32_t *col, uint32_t *newid,
                     uint8_t *present, uint64_t *out_rp, uint64_t *out_V, int threads)
{
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t v = 0; v < (int64_t)V0; v++) present[v] = rowptr[v + 1] > rowptr[v];
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t i = 0; i < (int64_t)E; i++) __atomic_store_n(&present[col[i]], (uint8_t)1, __ATOMIC_RELAXED);
    /* exclusive count of kept vertices: per-thread block sums, then a scan */
    uint64_t sums[1024];
    if (threads > 1023) threads = 1023;
    const uint64_t blk = (V0 + threads - 1) / threads;
#pragma omp parallel num_threads(threads)
    {
        const int t = omp_get_thread_num();
        const uint64_t b = t * blk, e = b + blk < V0 ? b + blk : V0;
        uint64_t s = 0;
        for (uint64_t v = b; v < e; v++) s += present[v];
        sums[t] = s;
#pragma omp barrier
#pragma omp single
        {
            uint64_t run = 0;
            for (int k = 0; k < omp_get_num_threads(); k++) {
                const uint64_t x = sums[k];
                sums[k] = run;
                run += x;
            }
            sums[omp_get_num_threads()] = run;
        }
        uint64_t id = sums[t];
        for (uint64_t v = b; v < e; v++) {
            newid[v] = (uint32_t)id;
            if (present[v]) out_rp[id++] = rowptr[v];
        }
#pragma omp barrier
#pragma omp single
        *out_V = sums[omp_get_num_threads()];
    }
    out_rp[*out_V] = E;
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t i = 0; i < (int64_t)E; i++) col[i] = newid[col[i]];
    return 0;
}
