// convert.cpp -- text edge list to a graph: the reference's converter_txt
// (tools/convert_from_txt.cc:66-218), as a library call.
//
// Default behaviour is the reference's:
//   - a line whose first character is not a digit is skipped (comments,
//     headers, blank lines, leading blanks: read_txt, :66-103);
//   - a line holds two unsigned ids; a self loop is dropped (:88-91);
//   - ids that appear in no edge are removed and the rest renumbered by rank,
//     keeping their order (remove_isolated_vertices, :105-140);
//   - every edge is added in both directions, the list sorted by (source,
//     destination) and duplicates removed (to_undirected, :142-166);
//   - V = number of vertices left, rowptr / col as the bcsr format holds them.
// Flags switch each step off (LT_EDGES_* in include/lighttraffic.h).  A line
// with fewer than two ids is skipped (the reference would reuse the previous
// line's destination); a file without edges is an error (the reference
// reads past an empty list).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "graph.h"

#ifdef _OPENMP
#include <parallel/algorithm>
#define LT_SORT __gnu_parallel::sort
#else
#define LT_SORT std::sort
#endif

namespace lt {

namespace {

inline bool is_digit(char c) { return c >= '0' && c <= '9'; }
inline bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Parse the edges of buf[0, n) (whole lines only); returns the offset of the
// first unconsumed byte.
size_t parse_lines(const char *buf, size_t n, bool last, int flags, std::vector<uint64_t> &src,
                   std::vector<uint64_t> &dst, uint64_t &max_id, bool &overflow)
{
    size_t i = 0;
    while (i < n) {
        const char *nl = static_cast<const char *>(std::memchr(buf + i, '\n', n - i));
        if (!nl && !last) break;
        const size_t end = nl ? (size_t)(nl - buf) : n;
        size_t k = i;
        if (k < end && is_digit(buf[k])) {
            uint64_t v[2] = {0, 0};
            int got = 0;
            while (got < 2 && k < end) {
                while (k < end && is_blank(buf[k])) k++;
                if (k >= end || !is_digit(buf[k])) break;
                uint64_t x = 0;
                while (k < end && is_digit(buf[k])) {
                    const uint64_t d = (uint64_t)(buf[k] - '0');
                    if (x > (UINT64_MAX - d) / 10) overflow = true;
                    x = x * 10 + d;
                    k++;
                }
                v[got++] = x;
            }
            if (got == 2 && (v[0] != v[1] || (flags & LT_EDGES_KEEP_SELF_LOOPS))) {
                src.push_back(v[0]);
                dst.push_back(v[1]);
                max_id = std::max(max_id, std::max(v[0], v[1]));
            }
        }
        i = nl ? end + 1 : n;
    }
    return i;
}

}  // namespace

lt_status read_edge_list(const char *path, int flags, lt_graph &g)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(LT_ERR_IO, "cannot open %s", path);
    std::vector<uint64_t> src, dst;
    uint64_t max_id = 0;
    bool overflow = false;
    std::vector<char> buf(64u << 20);
    size_t have = 0;
    for (;;) {
        const size_t r = std::fread(buf.data() + have, 1, buf.size() - have, f);
        have += r;
        const bool last = r == 0 || std::feof(f);
        const size_t used = parse_lines(buf.data(), have, last, flags, src, dst, max_id, overflow);
        std::memmove(buf.data(), buf.data() + used, have - used);
        have -= used;
        if (last && have == 0) break;
        if (last && used == 0) break;
        if (have == buf.size()) buf.resize(buf.size() * 2);  // a line longer than the buffer
    }
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return fail(LT_ERR_IO, "read error in %s", path);
    if (overflow) return fail(LT_ERR_FORMAT, "%s: a vertex id does not fit 64 bits", path);
    if (src.empty()) return fail(LT_ERR_FORMAT, "%s: no edges", path);

    // vertex ids: rank among the ids present (remove_isolated_vertices), or
    // the ids themselves
    const uint64_t n_raw = src.size();
    std::vector<uint32_t> s32(n_raw), d32(n_raw);
    uint64_t V = 0;
    if (flags & LT_EDGES_KEEP_ISOLATED) {
        if (max_id >= 0xFFFFFFFFull) return fail(LT_ERR_FORMAT, "%s: vertex id %llu does not fit 32 bits", path,
                                                (unsigned long long)max_id);
        for (uint64_t i = 0; i < n_raw; i++) {
            s32[i] = (uint32_t)src[i];
            d32[i] = (uint32_t)dst[i];
        }
        V = max_id + 1;
    } else {
        std::vector<uint64_t> ids(src);
        ids.insert(ids.end(), dst.begin(), dst.end());
        LT_SORT(ids.begin(), ids.end());
        ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
        if (ids.size() >= 0xFFFFFFFFull) return fail(LT_ERR_FORMAT, "%s: more than 2^32 - 1 vertices", path);
        V = ids.size();
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n_raw; i++) {
            s32[i] = (uint32_t)(std::lower_bound(ids.begin(), ids.end(), src[i]) - ids.begin());
            d32[i] = (uint32_t)(std::lower_bound(ids.begin(), ids.end(), dst[i]) - ids.begin());
        }
    }
    src.clear();
    src.shrink_to_fit();
    dst.clear();
    dst.shrink_to_fit();

    // (source, destination) keys, both directions unless directed; sorted,
    // duplicates removed unless kept
    const bool both = !(flags & LT_EDGES_DIRECTED);
    std::vector<uint64_t> key(both ? 2 * n_raw : n_raw);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n_raw; i++) {
        key[i] = ((uint64_t)s32[i] << 32) | d32[i];
        if (both) key[n_raw + i] = ((uint64_t)d32[i] << 32) | s32[i];
    }
    s32.clear();
    s32.shrink_to_fit();
    d32.clear();
    d32.shrink_to_fit();
    LT_SORT(key.begin(), key.end());
    if (!(flags & LT_EDGES_KEEP_DUPLICATES)) key.erase(std::unique(key.begin(), key.end()), key.end());

    g.V = (uint32_t)V;
    g.E = key.size();
    LT_TRY(host_alloc(g.rowptr_buf, 8ull * (V + 1), true));
    LT_TRY(host_alloc(g.col_buf, 4ull * g.E, true));
    uint64_t *rp = g.rowptr_mut();
    uint32_t *col = g.col_mut();
    std::memset(rp, 0, 8ull * (V + 1));
    for (uint64_t k = 0; k < g.E; k++) {
        rp[(key[k] >> 32) + 1]++;
        col[k] = (uint32_t)key[k];
    }
    for (uint64_t v = 0; v < V; v++) rp[v + 1] += rp[v];
    return LT_OK;
}

}  // namespace lt
