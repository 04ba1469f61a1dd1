// sched.cpp -- the plain (reference) and FIFO scheduling policies.
#include "sched.h"

#include <algorithm>

namespace lt {

bool Policy::next(const SchedView &v, int32_t prev_computed, bool sync, uint32_t &choice)
{
    uint64_t best = 0;
    bool picked = false;
    for (uint32_t i = 0; i < v.P; i++) {
        if ((int32_t)i == prev_computed && !sync) continue;
        if (v.waiting[i] > best) {
            best = v.waiting[i];
            choice = i;
            picked = true;
        }
    }
    return picked;
}

int32_t Policy::victim(const SchedView &v, int32_t except, uint32_t /*incoming*/)
{
    int32_t best = -1;
    for (uint32_t i = 0; i < v.P; i++) {
        if (v.slot_of[i] < 0 || (int32_t)i == except) continue;
        if (best < 0 || v.waiting[i] < v.waiting[best] ||
            (v.waiting[i] == v.waiting[best] && v.last_used[i] < v.last_used[best]))
            best = (int32_t)i;
    }
    return best;
}

// getComputedPartition (src/Scheduler.h:84-111): among cached partitions
// other than `except`, those with a full reference page on the device
// compete on the fewest walkers in total (device + host + not yet created);
// when none has one, the partition with the most device walkers.
int32_t Policy::overlap(const SchedView &v, int32_t except)
{
    int32_t full = -1, notfull = -1;
    for (uint32_t i = 0; i < v.P; i++) {
        if ((int32_t)i == except || v.slot_of[i] < 0) continue;
        const uint64_t on_gpu = v.dev[i];
        if (on_gpu >= kRefPageWalkers) {
            if (full < 0 || v.waiting[i] < v.waiting[full]) full = (int32_t)i;
        } else if (full < 0 && on_gpu > 0) {
            if (notfull < 0 || on_gpu > v.dev[notfull]) notfull = (int32_t)i;
        }
    }
    return full >= 0 ? full : notfull;
}

// FIFO variant (src/Scheduler.h:113-127): the first cached partition after
// `except` in cyclic order.  The reference would compute it even with an
// empty device queue (nothing to do until the copy ends); here such a pick
// ends the overlap.
int32_t FifoPolicy::overlap(const SchedView &v, int32_t except)
{
    const uint32_t start = except < 0 ? 0 : (uint32_t)except;
    for (uint32_t k = 1; k < v.P; k++) {
        const uint32_t i = (start + k) % v.P;
        if (v.slot_of[i] >= 0) return v.dev[i] > 0 ? (int32_t)i : -1;
    }
    return -1;
}

// FIFO_SCHE nextPartition (src/Scheduler.h:393-416): sweep partitions in id
// order, returning each one that has walkers; a finished sweep returns false
// once, after which the caller's outer loop starts the next sweep.
bool FifoPolicy::next(const SchedView &v, int32_t /*prev*/, bool /*sync*/, uint32_t &choice)
{
    if (cursor_ == 0) {
        bool any = false;
        for (uint32_t i = 0; i < v.P && !any; i++) any = v.waiting[i] > 0;
        if (!any) return false;
    }
    while (cursor_ < v.P) {
        choice = cursor_++;
        if (v.waiting[choice] > 0) return true;
    }
    cursor_ = 0;
    return false;
}

// FIFO victim (src/Scheduler.h:177-184): the first cached partition after the
// one loaded last, in cyclic id order.
int32_t FifoPolicy::victim(const SchedView &v, int32_t except, uint32_t /*incoming*/)
{
    const uint32_t start = except < 0 ? 0 : (uint32_t)except;
    for (uint32_t k = 1; k <= v.P; k++) {
        const uint32_t i = (start + k) % v.P;
        if ((int32_t)i != except && v.slot_of[i] >= 0) return (int32_t)i;
    }
    return -1;
}

}  // namespace lt
