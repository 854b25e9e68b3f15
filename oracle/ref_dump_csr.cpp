// TEST INFRASTRUCTURE ONLY.  Driver linked against the reference's own
// de-duplicating CSR loader (peel/src/graph.cpp:58-133, the loader behind
// peelone_dyn / peel_dyn), compiled from the reference sources where they lie
// by oracle/build_ref.sh.  Run it in an empty working directory that holds an
// `output/` folder: the loader writes its serialized cache there.  Output,
// little-endian binary: u32 V, u32 E, degrees[V], neighbors_offset[V+1],
// neighbors[E].
#include "graph.h"
#include <cstdio>

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: %s graph.mtx out.bin\n", argv[0]); return 2; }
    Graph g(argv[1]);
    FILE *f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    uint32_t hdr[2] = {g.V, g.E};
    std::fwrite(hdr, 4, 2, f);
    std::fwrite(g.degrees, 4, g.V, f);
    std::fwrite(g.neighbors_offset, 4, (size_t)g.V + 1, f);
    std::fwrite(g.neighbors, 4, g.E, f);
    std::fclose(f);
    return 0;
}
