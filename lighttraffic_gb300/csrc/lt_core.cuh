// lt_core.cuh -- types, the per-walker random stream and the three apps' step
// semantics, shared by every kernel of the engine.
//
// Random stream (replaces cuRAND XORWOW with per-thread state, src/Rand.h:1-37):
//   Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011)
//   key     = (seed lo32, seed hi32)
//   counter = (c0, tag | run << 8, walker index lo32, walker index hi32)
//     init draws: tag 1, c0 = draw number; step draws: tag 2, c0 = walker.step
//     before the update.  Every (walker, step) pair therefore owns one draw,
//     whatever thread, launch or schedule runs it.
//   r64 = x0 << 32 | x1 picks a neighbour or vertex as r64 % n (the integer
//   form of uniform_discrete_distribution, src/Rand.h:17-19);
//   m53 = (x2 << 32 | x3) >> 11 is the uniform double U = (m53 + 1) 2^-53 in
//   (0, 1]; the test U > p is done exactly in integers as m53 >= floor(p 2^53).
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#ifdef __CUDACC__
#define LT_HD __host__ __device__ __forceinline__
#else
#define LT_HD inline
#endif

namespace lt {

using nodeId = uint32_t;       // src/Type.h:5
using edgeId = uint64_t;       // src/Type.h:6
using walkId = uint64_t;       // src/Type.h:7
using partitionId = uint32_t;  // u16 in the reference (src/Type.h:8); the .part file keeps u16

constexpr nodeId kInvalidNode = 0xFFFFFFFFu;  // src/Type.h:18
constexpr uint32_t kTagInit = 1u;
constexpr uint32_t kTagStep = 2u;
constexpr uint32_t kTagRmatSrc = 0x10u;
constexpr uint32_t kTagRmatDst = 0x11u;

enum App : int { kPPR = 0, kPageRank = 1, kWalk = 2 };
enum Start : int { kStartSource = 0, kStartUniform = 1, kStartPerVertex = 2 };

struct Rand4 {
    uint32_t x0, x1, x2, x3;
};

LT_HD uint32_t mulhi32(uint32_t a, uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// Philox4x32 with 10 rounds.
LT_HD Rand4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
    constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t hi0 = mulhi32(M0, c0), lo0 = M0 * c0;
        const uint32_t hi1 = mulhi32(M1, c2), lo1 = M1 * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    return Rand4{c0, c1, c2, c3};
}

LT_HD Rand4 walk_draw(uint64_t seed, uint32_t c0, uint32_t tag, uint32_t run, uint64_t idx)
{
    return philox4x32_10(c0, tag | (run << 8), (uint32_t)idx, (uint32_t)(idx >> 32), (uint32_t)seed,
                         (uint32_t)(seed >> 32));
}

LT_HD uint64_t r64_of(const Rand4 &r) { return ((uint64_t)r.x0 << 32) | r.x1; }
LT_HD uint64_t m53_hi(const Rand4 &r) { return (((uint64_t)r.x0 << 32) | r.x1) >> 11; }
LT_HD uint64_t m53_of(const Rand4 &r) { return (((uint64_t)r.x2 << 32) | r.x3) >> 11; }

// floor(p * 2^53) for a float probability widened to double.
inline uint64_t threshold53(float p)
{
    const double d = (double)p;
    if (!(d > 0.0)) return 0;
    if (d >= 1.0) return (uint64_t)1 << 53;
    return (uint64_t)(d * 9007199254740992.0);
}

// x mod d for 0 < d < 2^16: long division in base 2^16 with three 32-bit
// remainders (every partial value stays below 2^32).
LT_HD uint32_t mod64_small(uint64_t x, uint32_t d)
{
    const uint32_t hi = (uint32_t)(x >> 32), lo = (uint32_t)x;
    uint32_t r = hi % d;
    r = ((r << 16) | (lo >> 16)) % d;
    r = ((r << 16) | (lo & 0xFFFFu)) % d;
    return r;
}

LT_HD float rcp_f32(float d)
{
#ifdef __CUDA_ARCH__
    return __frcp_rn(d);
#else
    return 1.0f / d;
#endif
}

// x mod d for 2^16 <= d < 2^32 without 64-bit division: reduce the high word
// (32-bit remainder), estimate the quotient of the remaining t = r1 2^32 + lo
// (t < d 2^32) in single precision, then correct in integers.  The estimate's
// relative error is below 2^-21, so after the first correction |r| < 1024 d;
// a second single-precision estimate of r / d (from r >> 16) leaves |r| < 3 d,
// which the final loops remove.  The result is exact whatever the rounding of
// the estimates.
LT_HD uint32_t mod64_large(uint64_t x, uint32_t d)
{
    const uint32_t hi = (uint32_t)(x >> 32), lo = (uint32_t)x;
    const uint32_t r1 = hi % d;
    const uint64_t t = ((uint64_t)r1 << 32) | lo;
    const float rd = rcp_f32((float)d);
    const float qf = ((float)r1 * 4294967296.0f + (float)lo) * rd;
    const uint32_t q = qf >= 4294967040.0f ? 0xFFFFFF00u : (qf <= 0.0f ? 0u : (uint32_t)qf);
    int64_t r = (int64_t)(t - (uint64_t)q * d);
    const int32_t c = (int32_t)floorf((float)(int32_t)(r >> 16) * 65536.0f * rd);
    r -= (int64_t)c * (int64_t)d;
    while (r < 0) r += d;
    while (r >= (int64_t)d) r -= d;
    return (uint32_t)r;
}

// r % n for the neighbour / vertex choice, without 64-bit division (which
// the compiler lowers through the FP64 pipe, slow on this part).  n fits 32
// bits on every graph the engine accepts (degree and V are below 2^32).
LT_HD uint64_t mod_u64(uint64_t r, uint64_t n)
{
    if ((n >> 32) == 0) {
        const uint32_t d = (uint32_t)n;
        return d <= 0xFFFFu ? mod64_small(r, d) : mod64_large(r, d);
    }
    return r % n;
}

// PPR walk length (src/walk/SingleSource.h:11-18): step = 2, then one more
// for every draw with U > prob.
LT_HD uint32_t ppr_length(uint64_t seed, uint32_t run, uint64_t idx, uint64_t thr)
{
    uint32_t step = 2;
    for (uint32_t t = 0;; t++) {
        const Rand4 r = walk_draw(seed, t, kTagInit, run, idx);
        if (m53_hi(r) < thr) return step;
        step++;
        if (m53_of(r) < thr) return step;
        step++;
    }
}

LT_HD uint32_t start_vertex(int start, uint32_t source, uint32_t V, uint64_t seed, uint32_t run, uint64_t idx)
{
    if (start == kStartSource) return source;
    if (start == kStartPerVertex) return (uint32_t)(idx % V);
    const Rand4 r = walk_draw(seed, 0, kTagInit, run, idx);
    return (uint32_t)mod_u64(r64_of(r), V);
}

// 16-bit lane l (0..7) of a Philox output, used by the RMAT generator.
LT_HD uint32_t lane16(const Rand4 &r, int l)
{
    const uint32_t w = (l >> 1) == 0 ? r.x0 : (l >> 1) == 1 ? r.x1 : (l >> 1) == 2 ? r.x2 : r.x3;
    return (l & 1) ? (w >> 16) : (w & 0xFFFFu);
}

}  // namespace lt
