// lt_cli.cpp -- the ppr / pagerank / genericwalk binaries.
//
// Built three times with LT_CLI_APP = 0 (ppr), 1 (pagerank), 2 (genericwalk).
// Accepts the reference's options (src/Config.h:40-52, readme.md "Options"):
//   -f/--file G.bcsr  -p/--partition P  -b/--batch B  -w/--walker W
//   -s/--partition-size MB  -l/--length L  --runs R  --trimmed T  --source v
//   --prob p  -m/--materialized-partition
// plus: --seed S, --start uniform|pervertex, --alpha a (PageRank teleport
// test, default 0.85 as app/pagerank.cu:6), --sched plain|fifo|learned|frequency|batched,
// --no-pipeline, --host-index (rowptr slices travel with the partitions,
// as in the reference), --zerocopy-threshold N, --counts-out FILE (u64[V] raw),
// --endpoints-out FILE / --paths-out FILE (genericwalk, u32 raw).
// Prints the reference's stdout lines (src/Config.h:92, src/LightTraffic.h:26,
// src/Scheduler.h:441-452, app/ppr.cu:107-110, app/pagerank.cu:232-248),
// including its "partitons" spelling, which benchmark scripts grep for.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lighttraffic.h"

#ifndef LT_CLI_APP
#define LT_CLI_APP 0
#endif

namespace {

struct Opts {
    std::string file;
    long long partitions = -1, batch = -1, walkers = -1, part_mb = 32, length = 10, runs = 1, trimmed = -1;
    long long source = 0;
    double prob = 0.15, alpha = 0.85;
    bool materialize = false;
    unsigned long long seed = 0x5EED5EEDull;
    int start = LT_START_UNIFORM;
    int sched = LT_SCHED_PLAIN;
    int pipeline = 1;
    int resident_index = 1;
    unsigned long long zc = UINT64_MAX;
    std::string counts_out, endpoints_out, paths_out;
    std::string checkpoint, resume;
    unsigned long long checkpoint_every = 100;
    bool checkpoint_stop = false;
};

[[noreturn]] void usage(const char *argv0, const char *msg)
{
    if (msg) fprintf(stderr, "%s\n", msg);
    fprintf(stderr,
            "usage: %s -f G.bcsr [-m] [-s MB] [-p P] [-b B] [-w W] [-l L] [--runs R] [--source v] [--prob p]\n"
            "          [--seed S] [--start uniform|pervertex] [--alpha a] [--sched plain|fifo|learned|frequency|batched]\n"
            "          [--no-pipeline] [--host-index] [--zerocopy-threshold N] [--counts-out F] [--endpoints-out F] [--paths-out F]\n"
            "          [--checkpoint F [--checkpoint-every N] [--stop-at-checkpoint]] [--resume F]\n",
            argv0);
    exit(2);
}

Opts parse(int argc, char **argv)
{
    Opts o;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i], val;
        bool has_eq = false;
        if (a.rfind("--", 0) == 0) {
            const size_t eq = a.find('=');
            if (eq != std::string::npos) {
                val = a.substr(eq + 1);
                a = a.substr(0, eq);
                has_eq = true;
            }
        }
        auto next = [&]() -> std::string {
            if (has_eq) return val;
            if (i + 1 >= argc) usage(argv[0], ("missing value for " + a).c_str());
            return argv[++i];
        };
        auto num = [&](const std::string &s) -> long long {
            char *end = nullptr;
            const long long v = strtoll(s.c_str(), &end, 10);
            if (!end || *end) {
                // the reference parses with istringstream, which accepts "1e9"-style input only as far as it
                // reads an integer; accept floating notation explicitly
                const double d = strtod(s.c_str(), &end);
                if (!end || *end) usage(argv[0], ("bad number: " + s).c_str());
                return (long long)d;
            }
            return v;
        };
        if (a == "-f" || a == "--file") o.file = next();
        else if (a == "-p" || a == "--partition") o.partitions = num(next());
        else if (a == "-b" || a == "--batch") o.batch = num(next());
        else if (a == "-w" || a == "--walker") o.walkers = num(next());
        else if (a == "-s" || a == "--partition-size") o.part_mb = num(next());
        else if (a == "-l" || a == "--length") o.length = num(next());
        else if (a == "--runs") o.runs = num(next());
        else if (a == "--trimmed") o.trimmed = num(next());
        else if (a == "--source") o.source = num(next());
        else if (a == "--prob") o.prob = atof(next().c_str());
        else if (a == "--alpha") o.alpha = atof(next().c_str());
        else if (a == "-m" || a == "--materialized-partition") o.materialize = true;
        else if (a == "--seed") o.seed = strtoull(next().c_str(), nullptr, 0);
        else if (a == "--start") {
            const std::string s = next();
            if (s == "uniform") o.start = LT_START_UNIFORM;
            else if (s == "pervertex") o.start = LT_START_PER_VERTEX;
            else usage(argv[0], "--start takes uniform or pervertex");
        } else if (a == "--sched") {
            const std::string s = next();
            if (s == "plain") o.sched = LT_SCHED_PLAIN;
            else if (s == "fifo") o.sched = LT_SCHED_FIFO;
            else if (s == "learned") o.sched = LT_SCHED_LEARNED;
            else if (s == "frequency") o.sched = LT_SCHED_FREQUENCY;
            else if (s == "batched") o.sched = LT_SCHED_BATCHED;
            else usage(argv[0], "--sched takes plain, fifo, learned, frequency or batched");
        } else if (a == "--no-pipeline") o.pipeline = 0;
        else if (a == "--host-index") o.resident_index = 0;
        else if (a == "--zerocopy-threshold") o.zc = strtoull(next().c_str(), nullptr, 0);
        else if (a == "--counts-out") o.counts_out = next();
        else if (a == "--endpoints-out") o.endpoints_out = next();
        else if (a == "--paths-out") o.paths_out = next();
        else if (a == "--checkpoint") o.checkpoint = next();
        else if (a == "--checkpoint-every") o.checkpoint_every = strtoull(next().c_str(), nullptr, 0);
        else if (a == "--stop-at-checkpoint") o.checkpoint_stop = true;
        else if (a == "--resume") o.resume = next();
        else if (a == "-h" || a == "--help") usage(argv[0], nullptr);
        else usage(argv[0], ("unknown option " + a).c_str());
    }
    if (o.file.empty()) usage(argv[0], "the -f option must be given");
    return o;
}

int die(lt_status s)
{
    fprintf(stderr, "error: %s: %s\n", lt_strerror(s), lt_last_error());
    return 1;
}

bool dump(const std::string &path, const void *p, size_t bytes)
{
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) return false;
    const bool ok = fwrite(p, 1, bytes, fp) == bytes;
    return fclose(fp) == 0 && ok;
}

}  // namespace

int main(int argc, char **argv)
{
    const Opts o = parse(argc, argv);
    lt_graph *g = nullptr;
    lt_status s = lt_graph_open(o.file.c_str(), o.materialize ? 1 : 0, (uint64_t)o.part_mb, &g);
    if (s != LT_OK) return die(s);
    lt_graph_info gi;
    lt_graph_info_get(g, &gi);
    lt_checkpoint_info ci{};
    if (!o.resume.empty()) {
        s = lt_checkpoint_read_info(o.resume.c_str(), &ci);
        if (s != LT_OK) return die(s);
        if (ci.app != LT_CLI_APP) {
            fprintf(stderr, "error: %s was written by another app\n", o.resume.c_str());
            return 1;
        }
    }
    const uint64_t W = !o.resume.empty() ? ci.num_walkers : o.walkers > 0 ? (uint64_t)o.walkers : 2ull * gi.num_nodes;
    printf("num nodes: %u, num edges: %lu, num walkers: %lu\n", gi.num_nodes, (unsigned long)gi.num_edges,
           (unsigned long)W);

    lt_engine_cfg cfg;
    lt_engine_cfg_default(&cfg);
    cfg.num_device_partitions = o.partitions > 0 ? (uint32_t)o.partitions : 0;
    cfg.num_device_walkers = o.batch > 0 ? (uint64_t)o.batch : 0;
    cfg.sched = o.sched;
    cfg.pipeline = o.pipeline;
    cfg.resident_index = o.resident_index;
    cfg.zerocopy_threshold = o.zc;
    cfg.seed = o.seed;
    lt_engine *e = nullptr;
    s = lt_engine_create(g, &cfg, &e);
    if (s != LT_OK) return die(s);
    const uint32_t cached = cfg.num_device_partitions ? cfg.num_device_partitions : gi.num_partitions;
    const uint64_t dev_walkers = cfg.num_device_walkers ? cfg.num_device_walkers : W;
    const int walker_bytes = LT_CLI_APP == 2 ? 12 : 12;
    printf("number of partitons: %u, graph memory pool: %lu MB, walker memory pool: %lu MB\n", gi.num_partitions,
           (unsigned long)(gi.partition_bytes * (cached < gi.num_partitions ? cached : gi.num_partitions) / 1024 / 1024),
           (unsigned long)(dev_walkers * walker_bytes / 1024 / 1024));

    if (!o.checkpoint.empty()) {
        s = lt_engine_checkpoint(e, o.checkpoint.c_str(), o.checkpoint_every, o.checkpoint_stop ? 1 : 0);
        if (s != LT_OK) return die(s);
    }
    std::vector<uint64_t> counts;
    const uint64_t *rowptr = nullptr;
    lt_graph_csr(g, &rowptr, nullptr);
#if LT_CLI_APP == 2
    std::vector<uint32_t> endpoints, paths;
    lt_stats acc{};
#endif
    if (!o.resume.empty()) {
        // finish the run saved in the checkpoint (one run for genericwalk)
#if LT_CLI_APP != 2
        counts.resize(gi.num_nodes);
        s = lt_resume(e, o.resume.c_str(), counts.data(), nullptr, nullptr);
#else
        endpoints.resize(ci.has_endpoints ? W : 0);
        paths.resize(ci.has_paths ? W * (uint64_t)(ci.length + 1) : 0);
        s = lt_resume(e, o.resume.c_str(), nullptr, endpoints.empty() ? nullptr : endpoints.data(),
                      paths.empty() ? nullptr : paths.data());
        if (s == LT_OK && !o.endpoints_out.empty() && !endpoints.empty() &&
            !dump(o.endpoints_out, endpoints.data(), 4 * endpoints.size()))
            fprintf(stderr, "cannot write %s\n", o.endpoints_out.c_str());
        if (s == LT_OK && !o.paths_out.empty() && !paths.empty() && !dump(o.paths_out, paths.data(), 4 * paths.size()))
            fprintf(stderr, "cannot write %s\n", o.paths_out.c_str());
        if (s == LT_OK) {
            printf("resumed run finished\n");
            lt_engine_destroy(e);
            lt_graph_close(g);
            return 0;
        }
#endif
    } else {
#if LT_CLI_APP == 0
    counts.resize(gi.num_nodes);
    s = lt_run_ppr(e, (uint32_t)o.source, W, (float)o.prob, counts.data());
#elif LT_CLI_APP == 1
    counts.resize(gi.num_nodes);
    s = lt_run_pagerank(e, W, (uint32_t)o.length, (uint32_t)o.runs, (float)o.alpha, o.start, counts.data());
#else
    endpoints.resize(o.endpoints_out.empty() ? 0 : W);
    paths.resize(o.paths_out.empty() ? 0 : W * (uint64_t)(o.length + 1));
    for (long long r = 0; r < o.runs && s == LT_OK; r++) {
        s = lt_run_walk(e, W, (uint32_t)o.length, (uint32_t)r, o.start, endpoints.empty() ? nullptr : endpoints.data(),
                        paths.empty() ? nullptr : paths.data());
        lt_stats st;
        lt_engine_stats(e, &st);
        acc.running_ms += st.running_ms;
        acc.iterations += st.iterations;
        acc.explicit_iterations += st.explicit_iterations;
        acc.graph_loading_ms += st.graph_loading_ms;
        acc.graph_loading_calls += st.graph_loading_calls;
        acc.computing_ms += st.computing_ms;
        acc.computing_calls += st.computing_calls;
    }
#endif
    }
    if (s == LT_INTERRUPTED) {
        printf("interrupted at checkpoint %s\n", o.checkpoint.c_str());
        return 4;
    }
    if (s != LT_OK) return die(s);
    lt_stats st;
    lt_engine_stats(e, &st);
#if LT_CLI_APP == 2
    st.running_ms = acc.running_ms;
    st.iterations = acc.iterations;
    st.explicit_iterations = acc.explicit_iterations;
    st.graph_loading_ms = acc.graph_loading_ms;
    st.graph_loading_calls = acc.graph_loading_calls;
    st.computing_ms = acc.computing_ms;
    st.computing_calls = acc.computing_calls;
#endif
    printf("Running Time: %f ms\n", st.running_ms);
    printf("iterations: %lu, explicit: %lu\n", (unsigned long)st.iterations, (unsigned long)st.explicit_iterations);
    printf("graph loading time: %f ms, calls: %lu\n", st.graph_loading_ms, (unsigned long)st.graph_loading_calls);
    printf("computing time: %f ms, calls: %lu\n", st.computing_ms, (unsigned long)st.computing_calls);
    printf("zero copy time: %f ms, calls: %lu\n", st.zerocopy_ms, (unsigned long)st.zerocopy_calls);
    printf("walker loading time: %f ms, calls: %lu\n", st.walker_loading_ms, (unsigned long)st.walker_loading_calls);
    printf("walker evicting time: %f ms, calls: %lu\n", st.walker_evicting_ms,
           (unsigned long)st.walker_evicting_calls);

    int rc = 0;
#if LT_CLI_APP == 0
    // app/ppr.cu:107-110
    const uint32_t target = 2;
    if (target < gi.num_nodes)
        printf("PageRank value of node %u: %f\n", target, (float)(counts[target] / (W / (gi.num_nodes + 0.0))));
    uint64_t sum = 0;
    for (uint64_t c : counts) sum += c;
    printf("sum: %lu, %lu\n", (unsigned long)sum, (unsigned long)W);
    printf(sum == W ? "result correct\n" : "result incorrect\n");
    rc = sum == W ? 0 : 3;
#elif LT_CLI_APP == 1
    // app/pagerank.cu:232-248
    auto result = [&](uint32_t i) {
        return (float)((counts[i] / (W * (double)o.runs / (gi.num_nodes + 0.0))) / (o.length + 0.0));
    };
    for (uint32_t i = 0, printed = 0; i < gi.num_nodes && printed < 20; i++) {
        const uint64_t deg = rowptr[i + 1] - rowptr[i];
        if (deg > 1000) {
            printf("node %u, degree %lu, value %f\n", i, (unsigned long)deg, result(i));
            printed++;
        }
    }
    printf("node 0, degree %lu, value %f\n", (unsigned long)rowptr[1], result(0));
    uint64_t sum = 0;
    for (uint64_t c : counts) sum += c;
    const uint64_t expected = W * (uint64_t)o.length * (uint64_t)o.runs;
    printf("sum: %lu, %lu\n", (unsigned long)sum, (unsigned long)expected);
    printf(sum == expected ? "result correct\n" : "result incorrect\n");
    rc = sum == expected ? 0 : 3;
#else
    if (!o.endpoints_out.empty() && !dump(o.endpoints_out, endpoints.data(), 4 * endpoints.size())) rc = 1;
    if (!o.paths_out.empty() && !dump(o.paths_out, paths.data(), 4 * paths.size())) rc = 1;
#endif
    if (!o.counts_out.empty() && !counts.empty() && !dump(o.counts_out, counts.data(), 8 * counts.size())) rc = 1;
    lt_engine_destroy(e);
    lt_graph_close(g);
    return rc;
}
