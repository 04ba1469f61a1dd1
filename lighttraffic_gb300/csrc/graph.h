// graph.h -- host-side graph: CSR in (pinned) host memory plus its vertex-range
// partition table.  Replaces DiskGraph/CPUGraph (src/GraphLoader.h:13-157) and
// PartitionStrategy (src/partition/PartitionStrategy.h:48-338).
#pragma once

#include <cstdint>
#include <vector>

#include "common.h"

struct lt_graph {
    uint32_t V = 0;
    uint64_t E = 0;
    lt::HostBuf rowptr_buf;  // u64[V+1]
    lt::HostBuf col_buf;     // u32[E]
    uint64_t part_bytes = 0;
    std::vector<uint32_t> node_off;  // P+1
    std::vector<uint64_t> edge_off;  // P+1
    uint32_t max_nodes = 0;
    uint64_t max_edges = 0;

    const uint64_t *rowptr() const { return (const uint64_t *)rowptr_buf.ptr; }
    const uint32_t *col() const { return (const uint32_t *)col_buf.ptr; }
    uint64_t *rowptr_mut() { return (uint64_t *)rowptr_buf.ptr; }
    uint32_t *col_mut() { return (uint32_t *)col_buf.ptr; }
    uint32_t P() const { return (uint32_t)node_off.size() - 1; }
    // Partition containing vertex v (binary search, PartitionStrategy.h:151-168).
    uint32_t find_partition(uint32_t v) const;
    // Device bytes of partition p's slot: rowptr slice (n+1 u64) then col slice.
    uint64_t slot_bytes(uint32_t p) const;
};

namespace lt {

lt_status partition_equal_size(const uint64_t *rowptr, uint32_t V, uint64_t max_bytes,
                               std::vector<uint32_t> &node_off, std::vector<uint64_t> &edge_off);
lt_status read_bcsr(const char *path, lt_graph &g);
// Text edge list -> CSR (tools/convert_from_txt.cc); flags LT_EDGES_*.
lt_status read_edge_list(const char *path, int flags, lt_graph &g);
lt_status write_bcsr(const lt_graph &g, const char *path);
lt_status read_part(const char *bcsr_path, lt_graph &g);
lt_status write_part(const lt_graph &g, const char *bcsr_path);
lt_status finish_partitions(lt_graph &g);  // fills max_nodes / max_edges, validates
void graph_free(lt_graph &g);

}  // namespace lt
