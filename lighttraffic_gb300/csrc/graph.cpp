// graph.cpp -- bcsr / .part files and the greedy partitioner.
#include "graph.h"

#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <string>

namespace lt {

namespace {
thread_local std::string g_last_error;
}

lt_status fail(lt_status s, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

void clear_error() { g_last_error.clear(); }
const char *last_error() { return g_last_error.c_str(); }

lt_status host_alloc(HostBuf &b, size_t bytes, bool want_pinned)
{
    host_free(b);
    size_t n = bytes ? bytes : 1;
    if (want_pinned) {
        int dev_count = 0;
        if (cudaGetDeviceCount(&dev_count) == cudaSuccess && dev_count > 0) {
            void *p = nullptr;
            if (cudaHostAlloc(&p, n, cudaHostAllocPortable | cudaHostAllocMapped) == cudaSuccess) {
                b.ptr = p;
                b.bytes = bytes;
                b.pinned = true;
                return LT_OK;
            }
            cudaGetLastError();
            return fail(LT_ERR_NOMEM, "cudaHostAlloc of %zu bytes failed", bytes);
        }
        cudaGetLastError();
    }
    void *p = nullptr;
    if (posix_memalign(&p, 4096, n) != 0 || !p) return fail(LT_ERR_NOMEM, "host allocation of %zu bytes failed", bytes);
    b.ptr = p;
    b.bytes = bytes;
    b.pinned = false;
    return LT_OK;
}

void host_free(HostBuf &b)
{
    if (b.ptr) {
        if (b.pinned)
            cudaFreeHost(b.ptr);
        else
            free(b.ptr);
    }
    b = HostBuf{};
}

// EqualSizeStrategy::init (src/partition/PartitionStrategy.h:193-218): grow the
// partition [n, i) while (i - n + 1) * 8 + (rowptr[i] - rowptr[n]) * 4 fits;
// when it stops fitting close the partition at i - 1 and test the same i
// again against the new start.  A single vertex that does not fit is an error.
lt_status partition_equal_size(const uint64_t *rowptr, uint32_t V, uint64_t max_bytes,
                               std::vector<uint32_t> &node_off, std::vector<uint64_t> &edge_off)
{
    node_off.assign(1, 0);
    edge_off.assign(1, 0);
    uint32_t n = 0;
    for (uint64_t i = 1; i <= V;) {
        const uint64_t size = (i - n + 1) * 8u + (rowptr[i] - rowptr[n]) * 4u;
        if (size > max_bytes) {
            if (i == (uint64_t)n + 1)
                return fail(LT_ERR_PARTITION, "Node %u has degree %llu. It cannot fit into partition size %llu", n,
                            (unsigned long long)(rowptr[i] - rowptr[n]), (unsigned long long)max_bytes);
            n = (uint32_t)(i - 1);
            node_off.push_back(n);
            edge_off.push_back(rowptr[n]);
        } else {
            i++;
        }
    }
    node_off.push_back(V);
    edge_off.push_back(rowptr[V]);
    return LT_OK;
}

lt_status finish_partitions(lt_graph &g)
{
    const uint32_t P = g.P();
    if (g.node_off.size() < 2 || g.node_off[0] != 0 || g.node_off[P] != g.V || g.edge_off[P] != g.E)
        return fail(LT_ERR_FORMAT, "partition table does not cover the graph");
    g.max_nodes = 0;
    g.max_edges = 0;
    for (uint32_t p = 0; p < P; p++) {
        if (g.node_off[p + 1] < g.node_off[p] || g.edge_off[p] != g.rowptr()[g.node_off[p]])
            return fail(LT_ERR_FORMAT, "partition %u is inconsistent with the graph", p);
        const uint32_t n = g.node_off[p + 1] - g.node_off[p];
        const uint64_t m = g.edge_off[p + 1] - g.edge_off[p];
        if (n > g.max_nodes) g.max_nodes = n;
        if (m > g.max_edges) g.max_edges = m;
    }
    return LT_OK;
}

namespace {

bool read_exact(FILE *fp, void *dst, size_t bytes)
{
    char *p = (char *)dst;
    while (bytes > 0) {
        const size_t chunk = bytes < (size_t(1) << 30) ? bytes : (size_t(1) << 30);
        const size_t got = fread(p, 1, chunk, fp);
        if (got != chunk) return false;
        p += got;
        bytes -= got;
    }
    return true;
}

bool write_exact(FILE *fp, const void *src, size_t bytes)
{
    const char *p = (const char *)src;
    while (bytes > 0) {
        const size_t chunk = bytes < (size_t(1) << 30) ? bytes : (size_t(1) << 30);
        if (fwrite(p, 1, chunk, fp) != chunk) return false;
        p += chunk;
        bytes -= chunk;
    }
    return true;
}

}  // namespace

// bcsr: u32 V | u64 E | u64 rowptr[V+1] | u32 col[E] (src/GraphLoader.h:30-48).
lt_status read_bcsr(const char *path, lt_graph &g)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(LT_ERR_IO, "cannot open %s: %s", path, strerror(errno));
    uint32_t V = 0;
    uint64_t E = 0;
    if (fread(&V, 4, 1, fp) != 1 || fread(&E, 8, 1, fp) != 1) {
        fclose(fp);
        return fail(LT_ERR_FORMAT, "%s: truncated bcsr header", path);
    }
    fseek(fp, 0, SEEK_END);
    const long long size = ftell(fp);
    const unsigned long long want = 12ull + 8ull * ((uint64_t)V + 1) + 4ull * E;
    if (size < 0 || (unsigned long long)size != want) {
        fclose(fp);
        return fail(LT_ERR_FORMAT, "%s: file has %lld bytes, header (V=%u, E=%llu) implies %llu", path, size, V,
                    (unsigned long long)E, want);
    }
    fseek(fp, 12, SEEK_SET);
    g.V = V;
    g.E = E;
    lt_status s = host_alloc(g.rowptr_buf, 8ull * ((uint64_t)V + 1), true);
    if (s == LT_OK) s = host_alloc(g.col_buf, 4ull * E, true);
    if (s != LT_OK) {
        fclose(fp);
        return s;
    }
    if (!read_exact(fp, g.rowptr_mut(), 8ull * ((uint64_t)V + 1)) || !read_exact(fp, g.col_mut(), 4ull * E)) {
        fclose(fp);
        return fail(LT_ERR_IO, "%s: short read", path);
    }
    fclose(fp);
    const uint64_t *rp = g.rowptr();
    if (rp[0] != 0 || rp[V] != E) return fail(LT_ERR_FORMAT, "%s: rowptr does not span [0, E]", path);
    for (uint64_t v = 0; v < V; v++)
        if (rp[v + 1] < rp[v]) return fail(LT_ERR_FORMAT, "%s: rowptr decreases at %llu", path, (unsigned long long)v);
    const uint32_t *c = g.col();
    for (uint64_t e = 0; e < E; e++)
        if (c[e] >= V) return fail(LT_ERR_FORMAT, "%s: col[%llu] = %u out of range", path, (unsigned long long)e, c[e]);
    return LT_OK;
}

lt_status write_bcsr(const lt_graph &g, const char *path)
{
    FILE *fp = fopen(path, "wb");
    if (!fp) return fail(LT_ERR_IO, "cannot create %s: %s", path, strerror(errno));
    const bool ok = fwrite(&g.V, 4, 1, fp) == 1 && fwrite(&g.E, 8, 1, fp) == 1 &&
                    write_exact(fp, g.rowptr(), 8ull * ((uint64_t)g.V + 1)) && write_exact(fp, g.col(), 4ull * g.E);
    if (fclose(fp) != 0 || !ok) return fail(LT_ERR_IO, "%s: write failed", path);
    return LT_OK;
}

// .part: u16 P | u64 partitionSize | u32 nodeOffset[P+1] | u64 edgeOffset[P+1]
// (written by materialize, src/partition/PartitionStrategy.h:325-337; read by
// MaterializedStrategy, :76-97).
lt_status read_part(const char *bcsr_path, lt_graph &g)
{
    const std::string path = std::string(bcsr_path) + ".part";
    FILE *fp = fopen(path.c_str(), "rb");
    if (!fp) return fail(LT_ERR_IO, "cannot open %s: %s (run with -m to create it)", path.c_str(), strerror(errno));
    uint16_t P = 0;
    uint64_t size = 0;
    bool ok = fread(&P, 2, 1, fp) == 1 && fread(&size, 8, 1, fp) == 1;
    if (ok && P == 0) ok = false;
    if (ok) {
        g.node_off.resize((size_t)P + 1);
        g.edge_off.resize((size_t)P + 1);
        ok = fread(g.node_off.data(), 4, (size_t)P + 1, fp) == (size_t)P + 1 &&
             fread(g.edge_off.data(), 8, (size_t)P + 1, fp) == (size_t)P + 1;
    }
    fclose(fp);
    if (!ok) return fail(LT_ERR_FORMAT, "%s: truncated partition file", path.c_str());
    g.part_bytes = size;
    LT_TRY(finish_partitions(g));
    for (uint32_t p = 0; p < g.P(); p++)
        if (g.slot_bytes(p) > size) return fail(LT_ERR_FORMAT, "%s: partition %u exceeds the partition size", path.c_str(), p);
    return LT_OK;
}

lt_status write_part(const lt_graph &g, const char *bcsr_path)
{
    const uint32_t P = g.P();
    if (P > 0xFFFFu) return fail(LT_ERR_INVALID, "%u partitions do not fit the u16 count of the .part format", P);
    const std::string path = std::string(bcsr_path) + ".part";
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) return fail(LT_ERR_IO, "cannot create %s: %s", path.c_str(), strerror(errno));
    const uint16_t P16 = (uint16_t)P;
    const bool ok = fwrite(&P16, 2, 1, fp) == 1 && fwrite(&g.part_bytes, 8, 1, fp) == 1 &&
                    fwrite(g.node_off.data(), 4, (size_t)P + 1, fp) == (size_t)P + 1 &&
                    fwrite(g.edge_off.data(), 8, (size_t)P + 1, fp) == (size_t)P + 1;
    if (fclose(fp) != 0 || !ok) return fail(LT_ERR_IO, "%s: write failed", path.c_str());
    return LT_OK;
}

void graph_free(lt_graph &g)
{
    host_free(g.rowptr_buf);
    host_free(g.col_buf);
}

}  // namespace lt

uint32_t lt_graph::find_partition(uint32_t v) const
{
    uint32_t lo = 0, hi = P() - 1;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (v < node_off[mid])
            hi = mid - 1;
        else
            lo = mid;
    }
    return lo;
}

uint64_t lt_graph::slot_bytes(uint32_t p) const
{
    return 8ull * ((uint64_t)(node_off[p + 1] - node_off[p]) + 1) + 4ull * (edge_off[p + 1] - edge_off[p]);
}
