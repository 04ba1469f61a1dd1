// ooc.h -- out-of-core run loop: partition cache, walker queues and scheduler.
//
// Replaces GPUScheduler / Scheduler (src/Scheduler.h:13-454), GPUGraph
// (src/GraphLoader.h:160-240), GPUListPool / ListPool (src/buffer/Pool.h:90-646)
// and GPUWalkManager (src/WalkManager.h:284-421) for graphs whose partitions
// do not all fit the device cache (-p smaller than the partition count).
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "common.h"
#include "sched.h"

struct lt_engine;
struct lt_server;

namespace lt {

struct Queue {
    std::vector<uint32_t> dev_chunks;   // all full except the last
    uint32_t tail_fill = 0;             // walkers in the last device chunk
    std::vector<uint32_t> host_chunks;  // spilled full chunks
    uint64_t lazy_next = 0;             // walkers created so far (lazy ordinals)
    uint64_t lazy_total = 0;

    uint64_t dev_count() const;
    uint64_t host_count() const;
    uint64_t lazy_left() const { return lazy_total - lazy_next; }
    uint64_t total() const { return dev_count() + host_count() + lazy_left(); }
};

struct Ooc;
lt_status ooc_create(lt_engine *e, Ooc **out);
void ooc_destroy(Ooc *o);
lt_status ooc_drop_cache(Ooc *o);
void ooc_policy_stats(const Ooc *o, lt_policy_stats &s);
lt_status ooc_autotune(lt_engine *e, lt_ooc_tune *out);
void ooc_partition_stats(const Ooc *o, uint64_t *visits, uint64_t *cached_visits, uint64_t *cached_launches);
lt_status ooc_run(lt_engine *e, int app, int start, uint32_t source, uint64_t W, uint32_t length, uint32_t runs,
                  uint32_t run_base, float prob, uint64_t *counts_out, uint32_t *endpoints_out, uint32_t *paths_out);

lt_status ooc_checkpoint(Ooc *o, const char *path, uint64_t every, int stop);
lt_status ooc_resume(lt_engine *e, const char *path, uint64_t *counts_out, uint32_t *endpoints_out,
                     uint32_t *paths_out);
lt_status checkpoint_info(const char *path, lt_checkpoint_info *out);

// Serving: PPR queries admitted, stepped and completed continuously.
lt_status serve_open(lt_engine *e, uint32_t max_active, uint64_t table_slots, float prob, lt_server **out);
lt_status serve_submit(lt_server *s, uint32_t source, uint64_t walkers, uint64_t seed, double arrival_ms,
                       uint64_t *ticket);
lt_status serve_step(lt_server *s, uint32_t *completed, uint32_t *active, uint32_t *pending);
lt_status serve_result(lt_server *s, uint64_t ticket, int *done, uint64_t *n_pairs, uint32_t *vertices,
                       uint32_t *counts, uint64_t capacity, double *latency_ms);
uint64_t serve_finished(lt_server *s, uint64_t *tickets, uint64_t cap);
void serve_close(lt_server *s);
double serve_now_ms();

}  // namespace lt
