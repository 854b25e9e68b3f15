// TEST INFRASTRUCTURE ONLY.  Driver of the reference's two peel/src GPU
// methods, int peel_dyn(Graph&) (peel/src/peel-dyn.cc:133-182) and
// int peelone_dyn(Graph&) (peel/src/peelone-dyn.cc:120-168), compiled
// unmodified from their sources with kcref_shim.h pre-included.  It replaces
// peel/main.cu:65-110, which times both methods ten times each and never
// reads the core numbers back: here one method runs once on the graph that
// the reference's own loader builds (Graph(std::string), peel/src/graph.cpp),
// and the device degrees array -- the core numbers when the method returns --
// is captured at its cudaFree and written as raw uint32 values.
//
// Usage: ref_dyn <graph.mtx> <peel_dyn|peelone_dyn> <core.bin>
// Prints "V: ...", "ms: ...", "kmax: ..." lines.  Run it in a fresh working
// directory holding an empty output/ folder (the loader caches its CSR there
// under the input's basename).
#include <stdio.h>
#include <sys/types.h>
#include <unistd.h>

#include "./inc/gpu_memory_allocation.h"
#include "./src/buffer.cc"
#include "./src/peel-dyn.cc"
#include "./src/peelone-dyn.cc"

int main(int argc, char *argv[]) {
    if (argc != 4) {
        fprintf(stderr, "usage: %s <graph.mtx> <peel_dyn|peelone_dyn> <core.bin>\n", argv[0]);
        return 2;
    }
    const std::string method = argv[2];
    if (method != "peel_dyn" && method != "peelone_dyn") {
        fprintf(stderr, "unknown method %s\n", argv[2]);
        return 2;
    }
    cudaFree(0);
    Graph g(argv[1]);
    printf("V: %u\n", g.V);
    kcref_track_host(g.degrees, (size_t)g.V * sizeof(unsigned int));
    const int ms = method == "peel_dyn" ? peel_dyn(g) : peelone_dyn(g);
    if (!kcref_state().have_capture) {
        fprintf(stderr, "core array was not captured\n");
        return 3;
    }
    FILE *f = fopen(argv[3], "wb");
    if (!f) return 4;
    fwrite(kcref_state().captured.data(), 1, kcref_state().captured.size(), f);
    fclose(f);
    printf("ms: %d\nkmax: %u\n", ms, g.kmax);
    return 0;
}
