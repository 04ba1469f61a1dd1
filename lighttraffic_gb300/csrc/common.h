// common.h -- status plumbing and host memory helpers shared by the host code.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "../../include/lighttraffic.h"

namespace lt {

// Records a message for lt_last_error() and returns s.
lt_status fail(lt_status s, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();
const char *last_error();

#define LT_CUDA_TRY(expr)                                                                    \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return ::lt::fail(LT_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #expr,        \
                              cudaGetErrorString(_e));                                       \
    } while (0)

#define LT_TRY(expr)                                                                         \
    do {                                                                                     \
        lt_status _s = (expr);                                                               \
        if (_s != LT_OK) return _s;                                                          \
    } while (0)

// Host allocation that is pinned when a CUDA device is usable (cudaHostAlloc,
// portable + mapped so zero-copy kernels can read it) and plain otherwise.
struct HostBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    bool pinned = false;
};
lt_status host_alloc(HostBuf &b, size_t bytes, bool want_pinned);
void host_free(HostBuf &b);

}  // namespace lt
