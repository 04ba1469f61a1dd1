// sched.h -- partition scheduling policies (host).
//
// The plain policy restates the reference scheduler (src/Scheduler.h):
//   next partition  = the one with the most waiting walkers, skipping the
//                     partition computed last unless nothing else waits
//                     (Scheduler::nextPartition, :368-388);
//   cache victim    = the cached partition with the fewest waiting walkers,
//                     other than the one loaded last
//                     (findPartitionwithleastWalker, :149-171); ties, which the
//                     reference breaks by unordered_map order, go to the
//                     partition loaded longest ago;
//   zero-copy       = a partition that is not cached and has fewer waiting
//                     walkers than the threshold is read over the host link
//                     (shouldZerocopy, :243-252).
// The FIFO policy restates the FIFO_SCHE variant (:113-127, :391-418).
// The learned policy (mlp.h) orders the same decisions by predicted arrivals.
#pragma once

#include <cstdint>
#include <vector>

namespace lt {

struct SchedView {
    uint32_t P = 0;
    const uint64_t *waiting = nullptr;   // P: walkers waiting per partition (device + host + not yet created)
    const int32_t *slot_of = nullptr;    // P: cache slot or -1
    const uint64_t *last_used = nullptr; // P: iteration the partition was last loaded or computed
    const uint32_t *arrivals = nullptr;  // P: walkers that arrived in the last iteration
    uint64_t iteration = 0;
};

class Policy {
public:
    virtual ~Policy() = default;
    // Scheduler::nextPartition: false when no partition has walkers.
    virtual bool next(const SchedView &v, int32_t prev_computed, bool sync, uint32_t &choice);
    // findPartitionwithleastWalker over cached partitions other than `except`; -1 if none.
    virtual int32_t victim(const SchedView &v, int32_t except, uint32_t incoming);
    // Partitions worth loading ahead of need (best first); plain: by waiting walkers.
    virtual void prefetch_order(const SchedView &v, uint32_t exclude, std::vector<uint32_t> &out);
    // Called after every iteration with the walkers that arrived per partition.
    virtual void observe(const SchedView &v) {}
    virtual const char *name() const { return "plain"; }
};

class FifoPolicy : public Policy {
    uint32_t cursor_ = 0;

public:
    bool next(const SchedView &v, int32_t prev_computed, bool sync, uint32_t &choice) override;
    int32_t victim(const SchedView &v, int32_t except, uint32_t incoming) override;
    const char *name() const override { return "fifo"; }
};

}  // namespace lt
