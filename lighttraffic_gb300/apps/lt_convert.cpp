// lt_convert.cpp -- the converter_txt binary: text edge list (.el) to .bcsr,
// invoked as the reference's tool is (readme.md "Datasets":
// `./converter_txt graph.el` writes graph.bcsr; tools/convert_from_txt.cc).
//   converter_txt GRAPH.el [--directed] [--keep-duplicates] [--keep-self-loops]
//                          [--keep-isolated]
// Without options the conversion is the reference's (lt_graph_from_edge_list).
#include <cstdio>
#include <cstring>
#include <string>

#include "lighttraffic.h"

int main(int argc, char **argv)
{
    std::string input;
    int flags = 0;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "--directed") flags |= LT_EDGES_DIRECTED;
        else if (a == "--keep-duplicates") flags |= LT_EDGES_KEEP_DUPLICATES;
        else if (a == "--keep-self-loops") flags |= LT_EDGES_KEEP_SELF_LOOPS;
        else if (a == "--keep-isolated") flags |= LT_EDGES_KEEP_ISOLATED;
        else if (input.empty() && a.size() && a[0] != '-') input = a;
        else {
            std::fprintf(stderr, "unknown argument %s\n", a.c_str());
            return 2;
        }
    }
    if (input.empty()) {
        std::fprintf(stderr, "usage: converter_txt GRAPH.el [--directed] [--keep-duplicates] [--keep-self-loops] "
                             "[--keep-isolated]\n");
        return 2;
    }
    if (input.size() < 3 || input.compare(input.size() - 3, 3, ".el") != 0) {
        std::fprintf(stderr, "Input file format is not supported (expects GRAPH.el).\n");
        return 2;
    }
    std::printf("read graph in text file...\n");
    lt_graph *g = nullptr;
    // one partition: the .part file is made when an app opens the graph (-m)
    lt_status s = lt_graph_from_edge_list(input.c_str(), flags, 1ull << 62, &g);
    if (s != LT_OK) {
        std::fprintf(stderr, "%s: %s\n", lt_strerror(s), lt_last_error());
        return 1;
    }
    lt_graph_info info;
    lt_graph_info_get(g, &info);
    std::printf("nodes: %u edges: %llu\n", info.num_nodes, (unsigned long long)info.num_edges);
    const std::string out = input.substr(0, input.size() - 2) + "bcsr";
    s = lt_graph_write_bcsr(g, out.c_str());
    lt_graph_close(g);
    if (s != LT_OK) {
        std::fprintf(stderr, "%s: %s\n", lt_strerror(s), lt_last_error());
        return 1;
    }
    return 0;
}
