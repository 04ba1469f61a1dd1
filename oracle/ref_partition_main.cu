// Harness around the reference's own host-side partitioner.
//
// TEST INFRASTRUCTURE ONLY: it is built from the reference sources in place
// (src/partition/PartitionStrategy.h, src/buffer/Buffer.h) into
// oracle/_ref/ref_partition and run on the CPU to produce golden .part files.
//
//   ref_partition <graph.bcsr> <max_bytes>
//
// Calls EqualSizeStrategy(FILE*, maxSize) (src/partition/PartitionStrategy.h:243-253)
// and materialize(filename) (:325-337), which writes <graph.bcsr>.part, then
// prints one line per partition: "<nodeOffset> <edgeOffset>".  A vertex that
// does not fit raises std::runtime_error (:201-205); the harness prints
// "ERROR <message>" and exits with status 3.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sstream>
#include <stdexcept>
#include "partition/PartitionStrategy.h"

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s graph.bcsr max_bytes\n", argv[0]);
        return 2;
    }
    FILE *fp = fopen(argv[1], "r");
    if (!fp) {
        fprintf(stderr, "cannot open %s\n", argv[1]);
        return 2;
    }
    size_t maxBytes = strtoull(argv[2], nullptr, 10);
    try {
        EqualSizeStrategy s(fp, maxBytes);
        s.materialize(argv[1]);
        for (unsigned i = 0; i <= s.numPartition(); i++)
            printf("%u %lu\n", s.nodeOffset(i), (unsigned long)s.edgeOffset(i));
    } catch (std::exception &e) {
        printf("ERROR %s\n", e.what());
        fclose(fp);
        return 3;
    }
    fclose(fp);
    return 0;
}
