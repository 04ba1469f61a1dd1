/*
 * oracle/ref_shim/LightTraffic.h -- host stand-ins for the GPU plumbing that
 * the reference's app sources (app/ppr.cu, app/pagerank.cu,
 * app/genericwalk.cu) include, so that their App::update functions compile
 * with g++, unchanged and in place, and run on the CPU inside the oracle's
 * reference harness (oracle/ref_apps_main.cpp).
 *
 * TEST INFRASTRUCTURE ONLY, like everything under oracle/.  Nothing here is
 * reference code: it declares just enough of the names the app files use
 * (types of src/Type.h:5-8, the random-number calls of src/Rand.h, buffers,
 * Config, the walk managers, LightTraffic) for their AppManager and main()
 * to compile; only App::update and App::terminated are ever called.
 *
 * Random numbers.  The reference draws from per-thread cuRAND state; the
 * harness replaces it, exactly like the oracle and the product, with the
 * Philox4x32-10 stream keyed by (seed, run, walker index, step value):
 * before each App::update the harness keys the state with the walker's step,
 * and the two calls the apps make read fixed lanes of that draw --
 * uniform_discrete_distribution the r64 of lanes (x0, x1) in the integer form
 * of src/Rand.h:17-19, curand_uniform_double the U = (m53 + 1) 2^-53 of lanes
 * (x2, x3) -- whatever order the app calls them in.
 */
#pragma once

#include <cassert>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#define __device__
#define __global__
#define __host__
#define __forceinline__ inline

typedef uint32_t nodeId;
typedef uint64_t edgeId;
typedef uint64_t walkId;
typedef uint16_t partitionId;

struct ShimRandState {
    uint32_t x[4];  /* the Philox draw of the current (walker, step) */
};
typedef ShimRandState GPURandState;
typedef ShimRandState curandState;

/* The harness runs one host thread: a plain add. */
inline unsigned int atomicAdd(unsigned int *a, unsigned int v)
{
    const unsigned int old = *a;
    *a = old + v;
    return old;
}

inline uint64_t uniform_discrete_distribution(GPURandState &s, nodeId n)
{
    return ((static_cast<uint64_t>(s.x[0]) << 32) | s.x[1]) % n;
}

inline double curand_uniform_double(GPURandState *s)
{
    const uint64_t m53 = ((static_cast<uint64_t>(s->x[2]) << 32) | s->x[3]) >> 11;
    return (double)(m53 + 1) * (1.0 / 9007199254740992.0);
}

template <typename T>
struct ShimPtr {
    T *p = nullptr;
    T *ptr() { return p; }
};

template <typename T>
struct GPUBuffer {
    std::vector<T> v;
    GPUBuffer(size_t n, int /*gpu*/ = 0) : v(n) {}
    T *ptr() { return v.data(); }
    template <typename B>
    void to(B &) {}
};

template <typename T>
struct CPUBuffer {
    std::vector<T> v;
    explicit CPUBuffer(size_t n) : v(n) {}
    CPUBuffer(size_t n, const T *p) : v(p, p + n) {}
    T &operator[](size_t i) { return v[i]; }
    T *ptr() { return v.data(); }
    template <typename B>
    void to(B &) {}
};

struct PartitionStrategy {
    nodeId n = 0;
    nodeId numNode() { return n; }
};

struct Config {
    PartitionStrategy *_partitions = nullptr;
    FILE *_file = nullptr;
    walkId _numWalker = 0;
    nodeId _source = 0;
    float _prob = 0.15f;
    int _runs = 1;
    nodeId _step = 0;
    Config(int, char **) {}
};

struct CUDAStream {};

template <typename Walker>
struct WalkManager {};

template <typename App, typename Walker>
struct GPUWalkManager {
    template <typename Init>
    void insert(Init &, WalkManager<Walker> &, CUDAStream &) {}
};

template <typename AppManager, typename App, typename Walker>
struct LightTraffic {
    struct Cpu {
        struct Graph {
            ShimPtr<edgeId> rowptr() { return ShimPtr<edgeId>(); }
        } _graph;
    };
    Cpu *_cpu = nullptr;
    LightTraffic(Config &, AppManager &) {}
    void start(AppManager &) {}
};
