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
//                     partition used longest ago;
//   zero-copy       = a partition that is not cached and has fewer waiting
//                     walkers than the threshold is read over the host link
//                     (shouldZerocopy, :243-252);
//   no look-ahead loads (the reference loads the partition it is about to
//                     compute, :173-213);
//   overlap           = while that load is on the copy engine, compute a
//                     cached partition: among those holding at least a
//                     reference page (167 936 walkers, src/Type.h:15) on the
//                     device the one with the fewest walkers in total, else
//                     the one with the most device walkers
//                     (getComputedPartition, :84-111, used at :194-208).
// The FIFO policy restates the FIFO_SCHE variant (:113-127, :391-418).
// The learned, frequency and batched policies run the engine in waves (see
// Policy::wave) and differ only in which cached partitions they give up.
#pragma once

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/lighttraffic.h"

namespace lt {

struct SchedView {
    uint32_t P = 0;
    uint32_t K = 0;                      // cache slots
    const uint64_t *waiting = nullptr;   // P: walkers waiting per partition (device + host + not yet created)
    const uint64_t *lazy = nullptr;      // P: of those, walkers not yet created
    const uint64_t *dev = nullptr;       // P: of those, walkers in device chunks
    const int32_t *slot_of = nullptr;    // P: cache slot or -1
    const uint64_t *last_used = nullptr; // P: iteration the partition was last loaded or computed
    const uint32_t *arrivals = nullptr;  // P: walkers queued at each partition in the last iteration
    const uint32_t *visits = nullptr;    // P: walkers that entered each partition (cached or not) in it
    uint64_t iteration = 0;
    uint64_t zc_threshold = 0;           // walkers below which a cold partition is read zero-copy
};

// Walkers in one page of the reference's device queues (numBlock x
// threadPerBlock x walkerPerThread, src/Type.h:10-15): the "full page" test
// of getComputedPartition.
constexpr uint64_t kRefPageWalkers = 82ull * 512 * 4;

class Policy {
public:
    virtual ~Policy() = default;
    // Scheduler::nextPartition: false when no partition has walkers.
    virtual bool next(const SchedView &v, int32_t prev_computed, bool sync, uint32_t &choice);
    // findPartitionwithleastWalker over cached partitions other than `except`; -1 if none.
    virtual int32_t victim(const SchedView &v, int32_t except, uint32_t incoming);
    // getComputedPartition: a cached partition other than `except` whose
    // device walkers to step while the load of `except` is in flight; -1 if
    // none.
    virtual int32_t overlap(const SchedView &v, int32_t except);
    // shouldZerocopy for a partition that is not cached.
    virtual bool zero_copy(const SchedView &v, uint32_t p, uint64_t threshold) { return v.waiting[p] < threshold; }
    // Called after every iteration; v.arrivals holds that iteration's arrivals.
    virtual void observe(const SchedView &v) {}
    // Wave runs: higher = better kept in the cache (victims have the lowest).
    virtual double cache_score(const SchedView &v, uint32_t p) { return 0.0; }
    // Wave runs: forecast walkers entering p per iteration, or < 0 when the
    // policy has no forecast (then the cache is never refilled by forecast).
    virtual double visit_rate(const SchedView &v, uint32_t p) { return -1.0; }
    // Wave runs: each step kernel drains every readable queue (all cached
    // partitions with walkers, plus a zero-copy set in the final phase) while
    // the loads for the next kernel run on the copy stream.  At most
    // wave_loads() loads start per kernel: the partitions not cached with the
    // most waiting walkers (at least the zero-copy threshold), into the slots
    // of idle cached partitions with the lowest cache_score (ties: least
    // recently used).
    virtual bool wave() const { return false; }
    virtual size_t wave_loads() const { return 8; }
    // Cache emptied (the learned state of a policy survives).
    virtual void reset() {}
    // A new run starts (its walkers are about to be created).
    virtual void run_start() {}
    // Wave runs, cold cache at a run's start: partitions to load into the
    // free slots before any walker queues, best first (false: none; the
    // slots then fill as walkers arrive).
    virtual bool prefill(const SchedView &v, std::vector<uint32_t> &order) { return false; }
    virtual void stats(lt_policy_stats &s) const
    {
        std::memset(&s, 0, sizeof s);
        std::strncpy(s.name, name(), sizeof s.name - 1);
    }
    virtual const char *name() const { return "plain"; }
};

// The plain policy's rules executed as wave runs (least recently used
// victims): separates what wave execution gains from what predictions gain.
class BatchedPolicy : public Policy {
public:
    bool wave() const override { return true; }
    const char *name() const override { return "batched"; }
};

class FifoPolicy : public Policy {
    uint32_t cursor_ = 0;

public:
    bool next(const SchedView &v, int32_t prev_computed, bool sync, uint32_t &choice) override;
    int32_t victim(const SchedView &v, int32_t except, uint32_t incoming) override;
    int32_t overlap(const SchedView &v, int32_t except) override;
    void reset() override { cursor_ = 0; }
    const char *name() const override { return "fifo"; }
};

}  // namespace lt
