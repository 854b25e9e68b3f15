// TEST INFRASTRUCTURE ONLY.  Driver linked against the reference's own COO
// loader and virtual-graph builder (index2core/shared/graph.cpp:17-95,
// virtual_graph.cpp:12-45,96-192), compiled from the reference sources where
// they lie by oracle/build_ref.sh.  It loads one MatrixMarket file exactly as
// the reference's HistoCore/NbrCore/CntCore/peelone/gppeel drivers do and
// writes the resulting arrays as little-endian binary for the golden-fixture
// generator:  u32 num_nodes, u32 num_edges, u32 hasZeroID, u32 Part_Size,
// u64 numParts, then edges (2*num_edges u32, 0-based), outDegree[num_nodes],
// nodePointer[num_nodes], edgeList[2*num_edges+num_nodes],
// partNodePointer[2*numParts].
#include "graph.h"
#include "virtual_graph.h"
#include <cstdio>

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: %s graph.mtx out.bin\n", argv[0]); return 2; }
    Graph graph(argv[1], false);
    graph.ReadGraph();
    VirtualGraph vg(graph, 64);
    vg.MakeUGraph();
    FILE *f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    uint32_t hdr[4] = {graph.num_nodes, graph.num_edges, graph.hasZeroID ? 1u : 0u, vg.Part_Size};
    std::fwrite(hdr, 4, 4, f);
    uint64_t np = (uint64_t)vg.numParts;
    std::fwrite(&np, 8, 1, f);
    for (uint32_t i = 0; i < graph.num_edges; i++) {
        uint32_t e[2] = {graph.edges[i].source, graph.edges[i].end};
        std::fwrite(e, 4, 2, f);
    }
    std::fwrite(vg.outDegree, 4, graph.num_nodes, f);
    std::fwrite(vg.nodePointer, 4, graph.num_nodes, f);
    std::fwrite(vg.edgeList, 4, (size_t)2 * graph.num_edges + graph.num_nodes, f);
    std::fwrite(vg.partNodePointer, 8, np, f);
    std::fclose(f);
    return 0;
}
