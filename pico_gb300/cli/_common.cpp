// Shared pieces of the CLI drivers: the reference's argument contract and
// report lines, over the C ABI of libkcore.so.
#include "_common.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace cli {

// argument::Parse / GenerateHelpString (index2core/shared/argument.cpp:36-107):
// exactly one argument (the input file), otherwise the help text and exit 0.
std::string parse_single_input(int argc, char **argv) {
    if (argc != 2) {
        std::string str = "\nRequired arguments:";
        str += "\n    [--input]: Input graph file. E.g., --input FacebookGraph.txt";
        str += "\nOptional arguments";
        str += "\n    [--output]: Output file for results. E.g., --output results.txt";
        str += "\n    [--device]: Select GPU device (default: 0). E.g., --device 1";
        str += "\n\n";
        std::printf("%s", str.c_str());
        std::exit(0);
    }
    return argv[1];
}

void die(const char *what) {
    std::fprintf(stderr, "%s: %s\n", what, kc_last_error());
    std::exit(1);
}

// Graph::ReadGraph's report (index2core/shared/graph.cpp:20,91-95) and the
// COO load + device build.
kc_graph *load_coo(const std::string &path) {
    std::printf("Reading the input graph from the following file:\n>> %s\n", path.c_str());
    uint32_t n = 0, *src = nullptr, *dst = nullptr;
    uint64_t m = 0;
    if (kc_parse_mtx(path.c_str(), KC_LOAD_COO, &n, &m, &src, &dst) != KC_OK) die("load");
    std::printf("Done reading.\n");
    std::printf("Number of nodes = %u\n", n);
    std::printf("Number of edges = %llu\n", (unsigned long long)m);
    kc_graph *g = nullptr;
    int rc = kc_graph_from_edges(src, dst, m, n, 0u, 0, &g);
    kc_host_free_edges(src, dst);
    if (rc != KC_OK) die("graph build");
    return g;
}

// Timed decomposition and the report of the index2core / peelone / gppeel
// drivers (e.g. HistoCore.cu:344-356, util.cpp:6-22).
int run_report(kc_graph *g, int method) {
    kc_stats st;
    uint32_t n = 0;
    kc_graph_info(g, &n, nullptr, nullptr, nullptr);
    std::vector<uint32_t> core(n ? n : 1);
    if (kc_decompose(g, method, core.data(), 0, &st, nullptr) != KC_OK) die("decompose");
    std::printf("Number of iterations = %u\n", st.iterations);
    std::printf("Processing finished in %g (ms).\n", st.ms);
    std::printf(" Max K = %u\n", st.kmax);
    std::printf(" Min K = %u\n", st.kmin);
    const char *out = std::getenv("KCORE_OUTPUT");
    if (out && *out) save_results(out, core.data(), n);
    kc_graph_free(g);
    return 0;
}

// utility::SaveResults (util.cpp:70-89): "i core" per line.
void save_results(const std::string &path, const uint32_t *core, uint32_t n) {
    std::printf("Saving the results into the following file:\n>> %s\n", path.c_str());
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", path.c_str());
        return;
    }
    for (uint32_t i = 0; i < n; i++) std::fprintf(f, "%u %u\n", i, core[i]);
    std::fclose(f);
    std::printf("Done saving.\n");
}

}  // namespace cli
