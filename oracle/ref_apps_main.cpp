/*
 * oracle/ref_apps_main.cpp -- the reference's own App::update, run on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle ref` into oracle/_ref/
 * (git-ignored) from the reference tree in place: app/ppr.cu, app/pagerank.cu
 * and app/genericwalk.cu are #included unchanged (REF_ROOT/app on the include
 * path), each inside its own namespace, against the host stand-ins of
 * oracle/ref_shim/ for the GPU plumbing they include.  Nothing of the
 * reference is copied into this repository.
 *
 * What runs is the reference's update code -- App::update and App::terminated
 * of each app -- driven the way its step kernel drives it
 * (src/WalkManager.h:229-246: `while (walker.step > 0 && walker.current in
 * [nodeBegin, nodeEnd)) rw->update(walker, rowptr, col, nodeBegin,
 * edgeBegin, state)` on the partition's rowptr and col slices), partition by
 * partition until every walker has finished.  The random stream is the keyed
 * Philox stream of the oracle and the product (see ref_shim/LightTraffic.h),
 * so the output must equal the oracle's bit for bit; that is how the
 * oracle's restatement of the three apps is pinned to the reference's code.
 * Initialisation is restated here: the geometric PPR length of
 * src/walk/SingleSource.h:11-18 (`step = 2; while (U > prob) step++`, U in
 * (0, 1] compared as a double, as curand_uniform_double is) and the uniform
 * start of src/walk/NodeSampler.h:10-13; their header files hold CUDA kernel
 * launches, which g++ cannot compile.
 *
 *   ref_apps APP GRAPH.bcsr PARTS START SOURCE W LENGTH PROB RUNS RUN0 SEED OUT
 *     APP    ppr | pagerank | walk
 *     PARTS  number of equal vertex ranges the walk is driven over
 *     START  0 source, 1 uniform, 2 per-vertex (walker i at vertex i mod V)
 *     OUT    ppr / pagerank: u64 counts[V]; walk: u32 endpoints[W], then
 *            u32 paths[W (LENGTH + 1)] (source + LENGTH hops, 0xFFFFFFFF
 *            after a vertex without out-edges)
 * A PageRank walker at a vertex without out-edges makes the reference
 * compute `% 0` (app/pagerank.cu:42); run PageRank only on graphs where
 * every vertex has out-edges.
 */
#include "LightTraffic.h"
#include "walk/NodeSampler.h"
#include "walk/SingleSource.h"

#include <cstring>
#include <string>

#define main ref_main_ppr
namespace ref_ppr {
#include "ppr.cu"
}
#undef main
#define main ref_main_pagerank
namespace ref_pagerank {
#include "pagerank.cu"
}
#undef main
#define main ref_main_genericwalk
namespace ref_genericwalk {
#include "genericwalk.cu"
}
#undef main

namespace {

constexpr uint32_t kTagInit = 1, kTagStep = 2;

/* Philox4x32-10 (Salmon et al., SC 2011), the stream of the oracle. */
void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t x[4])
{
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0;
        c1 = (uint32_t)p1;
        c2 = n2;
        c3 = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    x[0] = c0;
    x[1] = c1;
    x[2] = c2;
    x[3] = c3;
}

void key(GPURandState &s, uint64_t seed, uint32_t c0, uint32_t tag, uint32_t run, uint64_t idx)
{
    philox(c0, tag | (run << 8), (uint32_t)idx, (uint32_t)(idx >> 32), (uint32_t)seed, (uint32_t)(seed >> 32), s.x);
}

struct Graph {
    uint32_t V = 0;
    uint64_t E = 0;
    std::vector<uint64_t> rp;
    std::vector<uint32_t> col;
};

bool read_bcsr(const char *path, Graph &g)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    bool ok = std::fread(&g.V, 4, 1, f) == 1 && std::fread(&g.E, 8, 1, f) == 1;
    if (ok) {
        g.rp.resize((size_t)g.V + 1);
        g.col.resize(g.E);
        ok = std::fread(g.rp.data(), 8, g.rp.size(), f) == g.rp.size() &&
             (g.E == 0 || std::fread(g.col.data(), 4, g.E, f) == g.E);
    }
    std::fclose(f);
    return ok && g.rp[g.V] == g.E;
}

struct Run {
    int start;
    uint32_t source, length;
    float prob;
    uint64_t seed;
};

/* src/walk/SingleSource.h:11-18: trial j reads half j % 2 of init draw j / 2. */
uint32_t ppr_length(const Run &r, uint32_t run, uint64_t idx)
{
    uint32_t step = 2;
    GPURandState s;
    for (uint64_t j = 0;; j++) {
        key(s, r.seed, (uint32_t)(j / 2), kTagInit, run, idx);
        const uint64_t hi = j % 2 == 0 ? ((uint64_t)s.x[0] << 32) | s.x[1] : ((uint64_t)s.x[2] << 32) | s.x[3];
        const double u = (double)((hi >> 11) + 1) * (1.0 / 9007199254740992.0);
        if (!(u > (double)r.prob)) return step;
        step++;
    }
}

uint32_t start_vertex(const Run &r, uint32_t V, uint32_t run, uint64_t idx)
{
    if (r.start == 0) return r.source;
    if (r.start == 2) return (uint32_t)(idx % V);
    GPURandState s;
    key(s, r.seed, 0, kTagInit, run, idx);
    return (uint32_t)uniform_discrete_distribution(s, V);  /* src/walk/NodeSampler.h:11 */
}

/* Drive the app's update over equal vertex ranges until every walker is done. */
template <typename App, typename Walker>
void drive(App &app, const Graph &g, uint32_t parts, std::vector<Walker> &w, const Run &r, uint32_t run,
           uint32_t *paths)
{
    std::vector<uint32_t> noff(parts + 1);
    for (uint32_t p = 0; p <= parts; p++) noff[p] = (uint32_t)((uint64_t)g.V * p / parts);
    auto find = [&](uint32_t v) {
        uint32_t lo = 0, hi = parts - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (v < noff[mid]) hi = mid - 1; else lo = mid;
        }
        return lo;
    };
    std::vector<std::vector<uint64_t>> q(parts);
    for (uint64_t i = 0; i < w.size(); i++)
        if (w[i].step > 0) q[find(w[i].current)].push_back(i);
    for (bool any = true; any;) {
        any = false;
        for (uint32_t p = 0; p < parts; p++) {
            std::vector<uint64_t> mine;
            mine.swap(q[p]);
            const nodeId nb = noff[p], ne = noff[p + 1];
            const edgeId eb = g.rp[nb];
            for (uint64_t i : mine) {
                Walker &x = w[i];
                while (x.step > 0 && x.current >= nb && x.current < ne) {
                    GPURandState s;
                    const uint32_t step = x.step, cur = x.current;
                    key(s, r.seed, step, kTagStep, run, i);
                    app.update(x, g.rp.data() + nb, g.col.data() + eb, nb, eb, s);
                    if (paths) {
                        uint32_t *path = paths + i * ((uint64_t)r.length + 1);
                        if (g.rp[cur + 1] > g.rp[cur])
                            path[r.length - step + 1] = x.current;
                        else
                            for (uint32_t h = r.length - step + 1; h <= r.length; h++) path[h] = 0xFFFFFFFFu;
                    }
                }
                if (x.step > 0) {
                    q[find(x.current)].push_back(i);
                    any = true;
                }
            }
        }
    }
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 13) {
        std::fprintf(stderr, "usage: ref_apps APP GRAPH PARTS START SOURCE W LENGTH PROB RUNS RUN0 SEED OUT\n");
        return 2;
    }
    const std::string app = argv[1];
    Graph g;
    if (!read_bcsr(argv[2], g) || g.V == 0) {
        std::fprintf(stderr, "cannot read %s\n", argv[2]);
        return 1;
    }
    const uint32_t parts = (uint32_t)std::strtoul(argv[3], nullptr, 10);
    Run r;
    r.start = std::atoi(argv[4]);
    r.source = (uint32_t)std::strtoul(argv[5], nullptr, 10);
    const uint64_t W = std::strtoull(argv[6], nullptr, 10);
    r.length = (uint32_t)std::strtoul(argv[7], nullptr, 10);
    r.prob = std::strtof(argv[8], nullptr);
    const uint32_t runs = (uint32_t)std::strtoul(argv[9], nullptr, 10);
    const uint32_t run0 = (uint32_t)std::strtoul(argv[10], nullptr, 10);
    r.seed = std::strtoull(argv[11], nullptr, 0);
    if (parts == 0 || parts > g.V || runs == 0 || r.source >= g.V) {
        std::fprintf(stderr, "bad arguments\n");
        return 2;
    }
    FILE *out = std::fopen(argv[12], "wb");
    if (!out) return 1;
    if (app == "ppr" || app == "pagerank") {
        std::vector<nodeId> value(g.V, 0);
        for (uint32_t run = run0; run < run0 + runs; run++) {
            if (app == "ppr") {
                ref_ppr::App a{value.data(), g.V, W};
                std::vector<ref_ppr::Walker> w(W);
                for (uint64_t i = 0; i < W; i++) w[i] = ref_ppr::Walker{start_vertex(r, g.V, run, i), ppr_length(r, run, i)};
                drive(a, g, parts, w, r, run, nullptr);
            } else {
                /* app/pagerank.cu:6 compares U with its constant alpha; PROB must be 0.85 */
                ref_pagerank::App a{value.data(), g.V, W, r.length};
                std::vector<ref_pagerank::Walker> w(W);
                for (uint64_t i = 0; i < W; i++) w[i] = ref_pagerank::Walker{start_vertex(r, g.V, run, i), r.length};
                drive(a, g, parts, w, r, run, nullptr);
            }
        }
        std::vector<uint64_t> c(value.begin(), value.end());
        std::fwrite(c.data(), 8, c.size(), out);
    } else if (app == "walk") {
        ref_genericwalk::App a{g.V, r.length};
        std::vector<ref_genericwalk::Walker> w(W);
        std::vector<uint32_t> paths(W * ((uint64_t)r.length + 1), 0);
        for (uint64_t i = 0; i < W; i++) {
            w[i] = ref_genericwalk::Walker{start_vertex(r, g.V, run0, i), r.length, (uint32_t)i};
            paths[i * ((uint64_t)r.length + 1)] = w[i].current;
        }
        drive(a, g, parts, w, r, run0, paths.data());
        std::vector<uint32_t> ep(W);
        for (uint64_t i = 0; i < W; i++) ep[i] = w[i].current;
        std::fwrite(ep.data(), 4, ep.size(), out);
        std::fwrite(paths.data(), 4, paths.size(), out);
    } else {
        std::fprintf(stderr, "unknown app %s\n", app.c_str());
        return 2;
    }
    return std::fclose(out) == 0 ? 0 : 1;
}
